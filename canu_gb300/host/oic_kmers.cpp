// oic_kmers -- frequent k-mers of a read container on one GB300: the skip list that
// overlapInCore's -k <file> option reads.
//
//   oic_kmers -k 22 --min-count N [-h a-b] [--gpu-device d] -o ms22.dump reads.seqdb
//
// In canu this list comes from meryl (src/pipelines/canu/Meryl.pm: count the reads'
// canonical k-mers, print those at or above a threshold).  Output lines are
// "KMER<TAB>COUNT"; overlapInCore takes the first token of each line
// (overlapInCore-Build_Hash_Index.C:203-246).  The counting runs in liboic_gpu.so
// (oic_count_kmers).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "oic_gpu.h"
#include "oic_seqdb.h"

int main(int argc, char **argv) {
  uint32_t    K = 0, minCount = 0, bgn = 1, end = 0xffffffffu;
  int         device = 0, err = 0;
  const char *out = nullptr, *store = nullptr;
  for (int a = 1; a < argc; a++) {
    auto nxt = [&]() -> const char * { return a + 1 < argc ? argv[++a] : (err++, "0"); };
    if (!strcmp(argv[a], "-k")) K = (uint32_t)strtoul(nxt(), nullptr, 10);
    else if (!strcmp(argv[a], "--min-count")) minCount = (uint32_t)strtoul(nxt(), nullptr, 10);
    else if (!strcmp(argv[a], "-h")) {
      const char *v = nxt();
      char *e       = nullptr;
      bgn           = (uint32_t)strtoul(v, &e, 10);
      end           = (e && *e == '-') ? (uint32_t)strtoul(e + 1, nullptr, 10) : bgn;
    } else if (!strcmp(argv[a], "--gpu-device")) device = atoi(nxt());
    else if (!strcmp(argv[a], "-o")) out = nxt();
    else if (!store) store = argv[a];
    else {
      fprintf(stderr, "Unknown option '%s'\n", argv[a]);
      err++;
    }
  }
  if (err || !K || !minCount || !out || !store) {
    fprintf(stderr, "USAGE: %s -k K --min-count N [-h a-b] [--gpu-device d] -o out.dump reads.seqdb\n", argv[0]);
    return 1;
  }
  oic_seqdb db;
  if (oic_seqdb_load(store, &db)) {
    fprintf(stderr, "Failed to load read container '%s'\n", store);
    return 1;
  }
  oic_params P;
  oic_default_params(&P);
  P.kmerLen = K;
  oic_ctx *ctx = nullptr;
  int      rc  = oic_create(&P, device, &ctx);
  if (rc) {
    fprintf(stderr, "oic_create failed (%d): %s\n", rc, ctx ? oic_last_error(ctx) : "bad parameters or no CUDA device");
    return 1;
  }
  std::vector<uint32_t> lib(db.nReads), len(db.nReads);
  std::vector<uint64_t> off(db.nReads);
  for (uint32_t i = 0; i < db.nReads; i++) {
    lib[i] = db.index[i].libID;
    len[i] = db.index[i].length;
    off[i] = db.index[i].offset;
  }
  rc = oic_set_reads(ctx, db.nReads, lib.data(), len.data(), off.data(), db.bases, db.nBases);
  uint64_t n = 0;
  std::vector<char>     kmers;
  std::vector<uint32_t> counts;
  if (!rc) {
    rc = oic_count_kmers(ctx, bgn, end, minCount, nullptr, nullptr, 0, &n);
    if (rc == OIC_ERR_OVERFLOW) {   // sized: count again into room for n
      kmers.resize((size_t)n * K);
      counts.resize(n);
      rc = oic_count_kmers(ctx, bgn, end, minCount, kmers.data(), counts.data(), n, &n);
    }
  }
  if (rc) {
    fprintf(stderr, "oic_kmers failed (%d): %s\n", rc, oic_last_error(ctx));
    oic_destroy(ctx);
    return 1;
  }
  oic_destroy(ctx);
  FILE *F = fopen(out, "w");
  if (!F) {
    fprintf(stderr, "Failed to open '%s' for writing\n", out);
    return 1;
  }
  for (uint64_t i = 0; i < n; i++) fprintf(F, "%.*s\t%u\n", (int)K, kmers.data() + i * K, counts[i]);
  if (fclose(F)) return 1;
  fprintf(stderr, "%lu k-mers with count >= %u\n", (unsigned long)n, minCount);
  oic_seqdb_free(&db);
  return 0;
}
