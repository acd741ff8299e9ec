/* Stand-in for <cublas_v2.h>: the reference kernels use no cuBLAS symbol. */
#pragma once
#include "cuComplex.h"
