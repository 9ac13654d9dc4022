/* Minimal stand-in for the BLIS header, written for this repository: only the
 * type names that the reference's vendored Haswell microkernel sources use
 * in their signatures. Used solely to compile those sources into the oracle's
 * reference build (oracle/_ref); no BLIS code is involved. */
#ifndef MOMMS_ORACLE_BLIS_STUB_H
#define MOMMS_ORACLE_BLIS_STUB_H
#include <stdint.h>
typedef int64_t dim_t;
typedef int64_t inc_t;
typedef struct { float real, imag; } scomplex;
typedef struct { double real, imag; } dcomplex;
typedef struct { void* a_next; void* b_next; inc_t is_a, is_b; } auxinfo_t;
typedef struct cntx_s cntx_t;
#endif
