/* Part of the ALGLIB stand-in for the CPU oracle build; everything lives in interpolation.h. */
#pragma once
#include "interpolation.h"
