/* A plain C host binding libqsgb.so through include/qsgb.h: the calls a C
 * (or cgo / JNI / N-API) binding would make first, none of which needs a
 * GPU.  Prints one line per check and exits non-zero on the first failure. */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "qsgb.h"

static int fail(const char* what) {
  printf("FAIL %s\n", what);
  return 1;
}

int main(void) {
  if (qsgb_abi_version() < 2) return fail("abi version");
  printf("abi %d\n", qsgb_abi_version());
  const char* s = qsgb_status_string(QSGB_ERR_INVALID);
  if (!s || !strlen(s)) return fail("status string");
  printf("status %d: %s\n", QSGB_ERR_INVALID, s);
  /* argument errors come back as status codes before any CUDA call */
  double ptm[256] = {0};
  int st = qsgb_apply_ptm2(NULL, NULL, ptm, 4, 4, 4, 4, 1, 1, 1, QSGB_PTM_HOST, QSGB_F64, QSGB_ARITH_AUTO, 256,
                           NULL, NULL);
  if (st != QSGB_ERR_INVALID) return fail("null buffers");
  double a = 0, b = 0;
  st = qsgb_apply_ptm2(&a, &b, ptm, 0, 4, 4, 4, 1, 1, 1, QSGB_PTM_HOST, QSGB_F64, QSGB_ARITH_AUTO, 256, NULL,
                       NULL);
  if (st != QSGB_ERR_INVALID) return fail("zero dimension");
  st = qsgb_apply_ptm1(&a, &b, ptm, 4, 4, 1, 1, QSGB_PTM_HOST, 7, QSGB_ARITH_AUTO, 16, NULL, NULL);
  if (st != QSGB_ERR_INVALID) return fail("bad dtype");
  if (qsgb_marginals_noalloc_max_scratch_bytes() <= 0) return fail("scratch size");
  printf("argument checks ok\n");
  return 0;
}
