/* Stand-in for <cufft.h>: only the complex type the reference kernels use. */
#pragma once
#include "cuComplex.h"
typedef cuComplex cufftComplex;
