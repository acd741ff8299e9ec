/* Stand-in for <cuComplex.h>: single-precision complex as an 8-byte {x, y}. */
#pragma once
typedef struct __attribute__((aligned(8))) { float x, y; } cuComplex;
