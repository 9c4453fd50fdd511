// oic_merge -- merges the outputs of independent overlapInCore jobs into one.
//
//   oic_merge out.ovb job1.ovb job2.ovb ...
//
// canu splits the overlap stage into jobs of one hash block range against one ref
// range (src/overlapInCore/overlapInCorePartition.C:225-245); their records are
// disjoint.  The merged .ovb holds every job's snappy blocks in argument order (each
// block stands alone, so the file reads like one job's), and out.oc holds the sum of
// the jobs' .oc counts, read by read.  Exit status 0 on success, 1 on any failure.
#include <cerrno>
#include <cstdio>
#include <cstring>

#include "oic_ovfile.h"

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s out.ovb in1.ovb [in2.ovb ...]\n", argv[0]);
    return 1;
  }
  const int rc = oic_merge_outputs(argv[1], (const char *const *)(argv + 2), (uint32_t)(argc - 2));
  if (rc) {
    fprintf(stderr, "oic_merge: %s\n", rc == 1 ? strerror(errno) : "an input is not a framed .ovb with its .oc");
    return 1;
  }
  return 0;
}
