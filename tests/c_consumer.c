/* c_consumer.c -- test program: the library used from plain C99 through its public
 * headers, as an FFI binding (cgo, JNI, ctypes) sees it.  Run by tests/test_c_consumer.py
 * on a host with or without a GPU: the host-only entry points must work, and context
 * creation must either succeed (a GPU is present) or return OIC_ERR_CUDA cleanly.
 *
 *   c_consumer <scratch dir>      prints "ok create=<code>" and exits 0 on success */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "oic_gpu.h"
#include "oic_ovfile.h"
#include "oic_seqdb.h"

static int fail(const char *what) {
  fprintf(stderr, "c_consumer: %s\n", what);
  return 1;
}

int main(int argc, char **argv) {
  char        path[4096], oc[4096], json[4096];
  oic_params  p;
  oic_stats   st;
  oic_ctx    *ctx = NULL;
  uint32_t    rec[2 * 6] = {1, 2, 0, 5, 0, 0, 2, 1, 0, 3, 0, 0};
  uint32_t    back[2 * 6];
  uint32_t    lens[2] = {1000, 2000};
  uint64_t    n = 0;
  size_t      len = 0;
  int         rc;
  if (argc != 2) return 2;

  oic_default_params(&p);

  memset(&st, 0, sizeof(st));
  st.totalOverlaps = 10;
  st.msTotal       = 1000.0;
  if (oic_stats_json(&st, json, sizeof(json), &len) != OIC_OK || len != strlen(json) ||
      !strstr(json, "\"overlapsPerSec\": 10.000"))
    return fail("oic_stats_json");

  snprintf(path, sizeof(path), "%s/job.ovb", argv[1]);
  if (oic_ovb_write(path, rec, 2, 1) != 0) return fail("oic_ovb_write");
  if (oic_ovb_read(path, back, 2, &n) != 0 || n != 2 || memcmp(rec, back, sizeof(rec)) != 0)
    return fail("oic_ovb_read");
  if (oic_oc_path(path, oc, sizeof(oc)) != 0 || oic_oc_write(oc, rec, 2, 2) != 0) return fail("oic_oc_write");

  /* store records sorted: (1, 2, ...) then (2, 1, ...) */
  snprintf(path, sizeof(path), "%s/asm.ovlStore", argv[1]);
  if (oic_ovstore_write(path, rec, 2, lens, 2, 0) != 0) return fail("oic_ovstore_write");

  p.kmerLen = 22;   /* valid parameters, so that creation reaches the device */
  rc = oic_create(&p, 0, &ctx);
  if (rc == OIC_OK) {
    oic_destroy(ctx);
  } else if (rc != OIC_ERR_CUDA) {
    return fail("oic_create returned an unexpected code");
  }
  printf("ok create=%d\n", rc);
  return 0;
}
