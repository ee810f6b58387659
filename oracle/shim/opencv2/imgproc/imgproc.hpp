/* Part of the OpenCV stand-in for the CPU oracle build; everything lives in core.hpp. */
#pragma once
#include "../core.hpp"
