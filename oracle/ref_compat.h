/* ref_compat.h — TEST INFRASTRUCTURE ONLY.  Force-included (g++ -include) by
 * oracle/build_ref.py when it compiles the reference's sources: the MSVC
 * runtime names the reference's PVM reader uses (fopen_s, sscanf_s,
 * errno_t; libs/file_utils/pvm.cpp) mapped to their standard C equivalents,
 * so the unmodified source builds with GCC. */
#ifndef CVR_REF_COMPAT_H
#define CVR_REF_COMPAT_H
#include <errno.h>
#include <stdio.h>
typedef int errno_t;
static inline errno_t fopen_s(FILE** f, const char* name, const char* mode) {
  *f = fopen(name, mode);
  return *f ? 0 : errno;
}
#define sscanf_s sscanf
#endif
