/* Type shim for compiling the reference general-XRCC C kernels (density_tensors.c,
 * H_contractions.c) outside of the Qode library, which normally supplies PyC_types.h.
 * Test infrastructure only: the compiled reference kernels are used as a CPU checker
 * and as the timed CPU baseline, never by the product path.
 * Qode's PyC maps PyInt/BigInt to 64-bit integers and Double/PyFloat to IEEE double. */
#ifndef XRH_ORACLE_PYC_TYPES_SHIM_H
#define XRH_ORACLE_PYC_TYPES_SHIM_H
typedef long long PyInt;
typedef long long BigInt;
typedef double    Double;
typedef double    PyFloat;
#endif
