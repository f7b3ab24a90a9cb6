/*
 * CPU oracle of the FDTD hot path, in float32 (the reference's storage precision) and
 * float64 (the same equations with every word in double).
 *
 * TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * arm load this library to check or time the CUDA engine; the product never links it.
 * Build: oracle/Makefile (gcc -O2 -ffp-contract=off, no fast-math: every operation
 * rounds once, like the reference's NumPy ufuncs).
 */
#include <math.h>
#include <stddef.h>

#define REAL float
#define SUF(x) x##_f32
#define NARROW(v) ((float)(v))
#include "fdtd_oracle_impl.h"
#undef REAL
#undef SUF
#undef NARROW

#define REAL double
#define SUF(x) x##_f64
#define NARROW(v) ((double)(v))
#include "fdtd_oracle_impl.h"
#undef REAL
#undef SUF
#undef NARROW

int oracle_abi_version(void) { return 1; }
