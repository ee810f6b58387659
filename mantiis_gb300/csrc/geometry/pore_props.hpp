// GPU pipeline of Shape::calculateProperties (include/shape.hpp:127-251).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <exception>

namespace mantiis
{
// largest image side the pipeline accepts (about 7.5 GB of device memory)
constexpr int kMaxPorePropsSide = 16384;

// Local pore size and Knudsen number of an n x n row-major 0/1 image (host
// pointers in and out); `iterations` (may be null) receives the number of
// thinning iterations up to and including the first that deleted nothing.
// Throws std::invalid_argument on bad arguments and a runtime_error on CUDA
// errors (is_geometry_cuda_error tells which).
void gpu_pore_properties(const int32_t *pore, int n, double dx, double mfp, double *locpore, double *kn,
                         int64_t *iterations, cudaStream_t stream);
bool is_geometry_cuda_error(const std::exception &e);
} // namespace mantiis
