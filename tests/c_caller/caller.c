/* A plain C99 caller of libskewgpu.so through include/skewgpu.h: what a Julia
 * ccall or any C host binds.  It creates a handle; on a machine without a GPU
 * that must fail with a status (not a crash), which is all it checks there.
 * Exit code: 0 when every call returned a status, 1 otherwise. */
#include <stdio.h>
#include <string.h>

#include "skewgpu.h"

int main(void) {
  printf("version %d\n", skew_version());
  skew_handle_t h = NULL;
  const int st = skew_create(&h);
  printf("skew_create -> %d (%s)\n", st, skew_status_string(st));
  if (st == SKEW_OK) {
    /* a bad argument is rejected on the host, before any launch */
    const int bad = skew_logabspf_d(h, NULL, 4, 4, NULL, NULL, 0, NULL);
    printf("skew_logabspf_d(NULL) -> %d (%s)\n", bad, skew_status_string(bad));
    skew_destroy(h);
    return bad == SKEW_BAD_ARG ? 0 : 1;
  }
  return (st == SKEW_CUDA_ERROR || st == SKEW_UNSUPPORTED) ? 0 : 1;
}
