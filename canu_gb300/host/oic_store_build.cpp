// oic_store_build -- the overlap-store build's record pass on the GPU.
//
//   oic_store_build -O out -S reads.seqdb [-e maxErate] [--store dir.ovlStore] [--gpu-device d]
//                   in1.ovb [in2.ovb ...]
//
// canu's ovStoreBuild (src/stores/ovStoreBuild.C) reads the overlapper's .ovb files,
// filters them (ovStoreFilter), adds every overlap's ID-swapped copy, sorts the kept
// records by (a_iid, b_iid, data) and writes them into the overlap store read by read.
// This tool does the reading, filtering, copying and sorting (oic_store_sort) and
// writes:
//   out.ovb    the sorted records, in ovFile's snappy-framed full-record format;
//   out.index  uint64 per read ID 0..maxID + 1: the index of the read's first record as
//              the a read (the last entry is the record count), i.e. each read's slice.
//   --store    also the overlap-store directory canu's own store writer makes from those
//              records (info, index, data files 0001-NNN, statistics; oic_ovstore_write),
//              which canu's ovStore reader opens.
// It prints the filter summary ovStoreBuild prints (ovStoreBuild.C:222-240).
// Differences: the inputs are listed on the command line (canu passes a store
// configuration file, -C).  Exit status 0 on success, 1 on any failure.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "oic_gpu.h"
#include "oic_ovfile.h"
#include "oic_seqdb.h"

int main(int argc, char **argv) {
  const char              *outName = nullptr, *seqName = nullptr, *storeDir = nullptr;
  double                   maxErate = 1.0;
  int                      device   = 0;
  std::vector<const char *> inputs;
  for (int a = 1; a < argc; a++) {
    if (!strcmp(argv[a], "-O") && a + 1 < argc) outName = argv[++a];
    else if (!strcmp(argv[a], "-S") && a + 1 < argc) seqName = argv[++a];
    else if (!strcmp(argv[a], "-e") && a + 1 < argc) maxErate = atof(argv[++a]);
    else if (!strcmp(argv[a], "--store") && a + 1 < argc) storeDir = argv[++a];
    else if (!strcmp(argv[a], "--gpu-device") && a + 1 < argc) device = atoi(argv[++a]);
    else if (argv[a][0] == '-') {
      fprintf(stderr, "%s: unknown option '%s'.\n", argv[0], argv[a]);
      return 1;
    } else inputs.push_back(argv[a]);
  }
  if (!outName || !seqName || inputs.empty()) {
    fprintf(stderr,
            "usage: %s -O out -S reads.seqdb [-e maxErate] [--store dir.ovlStore] [--gpu-device d] in1.ovb "
            "[in2.ovb ...]\n",
            argv[0]);
    return 1;
  }
  oic_seqdb db;
  if (oic_seqdb_load(seqName, &db)) {
    fprintf(stderr, "Failed to load read container '%s'\n", seqName);
    return 1;
  }
  const uint32_t        maxID = db.nReads;
  std::vector<uint32_t> readLen(maxID);
  for (uint32_t i = 0; i < maxID; i++) readLen[i] = db.index[i].length;
  oic_seqdb_free(&db);

  std::vector<uint32_t> words;
  for (const char *in : inputs) {
    uint64_t n = 0;
    if (oic_ovb_read(in, nullptr, 0, &n)) {
      fprintf(stderr, "Failed to read '%s'\n", in);
      return 1;
    }
    const size_t at = words.size();
    words.resize(at + n * 6);
    if (oic_ovb_read(in, words.data() + at, n, &n)) {
      fprintf(stderr, "Failed to read '%s'\n", in);
      return 1;
    }
    fprintf(stderr, "%12.3f Moverlaps %s\n", n / 1e6, in);
  }
  const uint64_t        nIn = words.size() / 6;
  std::vector<uint32_t> out(2 * nIn * 6 + 6);
  std::vector<uint64_t> perRead((size_t)maxID + 2);
  uint64_t              counts[5], nOut = 0;
  const int rc = oic_store_sort(device, words.data(), nIn, maxID, maxErate, out.data(), &nOut, perRead.data(), counts);
  if (rc) {
    fprintf(stderr, "oic_store_sort failed (%d)%s\n", rc,
            rc == OIC_ERR_INPUT ? ": an overlap has IDs out of range, possibly corrupt input data" : "");
    return 1;
  }
  fprintf(stderr, "\n-- OVERLAP FILTERING --\n\nTRIMMING OVERLAPS\n");
  fprintf(stderr, "Saved      %llu trimming overlaps\n", (unsigned long long)counts[1]);
  fprintf(stderr, "Discarded  %llu don't care\n\nUNITIGGING OVERLAPS\n", (unsigned long long)counts[3]);
  fprintf(stderr, "Saved      %llu unitigging overlaps\n\n", (unsigned long long)counts[0]);
  fprintf(stderr, "Discarded  %llu low quality, more than %.4f fraction error\n", (unsigned long long)counts[2],
          maxErate);
  fprintf(stderr, "Discarded  %llu opposite orientation\n\n", (unsigned long long)counts[4]);

  const std::string ovb = std::string(outName) + ".ovb", idx = std::string(outName) + ".index";
  if (oic_ovb_write(ovb.c_str(), out.data(), nOut, 1)) {
    fprintf(stderr, "Failed to write '%s': %s\n", ovb.c_str(), strerror(errno));
    return 1;
  }
  FILE *F = fopen(idx.c_str(), "wb");
  bool  ok = F && fwrite(perRead.data(), 8, perRead.size(), F) == perRead.size();
  ok       = (F && fclose(F) == 0) && ok;
  if (!ok) {
    fprintf(stderr, "Failed to write '%s': %s\n", idx.c_str(), strerror(errno));
    return 1;
  }
  if (storeDir) {
    const int wr = oic_ovstore_write(storeDir, out.data(), nOut, readLen.data(), maxID, 0);
    if (wr) {
      fprintf(stderr, "Failed to write the overlap store '%s'%s%s\n", storeDir, wr == 1 ? ": " : "",
              wr == 1 ? strerror(errno) : ": records out of order or outside the reads");
      return 1;
    }
    fprintf(stderr, "Created ovStore '%s' with %llu overlaps.\n", storeDir, (unsigned long long)nOut);
  }
  fprintf(stderr, "%llu overlaps in %s; index %s\nBye.\n", (unsigned long long)nOut, ovb.c_str(), idx.c_str());
  return 0;
}
