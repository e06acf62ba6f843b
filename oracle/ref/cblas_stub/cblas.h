/* Minimal stand-in for <cblas.h>: the reference's mdarray.hpp needs only the
 * layout enum (mdarray.hpp:27-35); no BLAS routine is called on the collocate
 * path.  Enum values follow the CBLAS standard. */
#ifndef GPW_ORACLE_CBLAS_STUB_H
#define GPW_ORACLE_CBLAS_STUB_H
typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
#endif
