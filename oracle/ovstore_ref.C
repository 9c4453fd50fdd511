/* ovstore_ref.C -- test infrastructure only: canu's own overlap-store writer and reader,
 * as the checker of the engine's ovStore directory writer.
 *
 * canu's src/stores/ovOverlap.C, ovStoreFile.C, ovStoreHistogram.C, ovStoreWriter.C and
 * ovStore.C are compiled where they lie: this file includes them by path (REF_*_C, set
 * by oracle/Makefile.ovstore), after oracle/shim_ovs/ovs_shim.H has provided the
 * meryl-utility file routines and a read-length store.
 *
 *   ovstore_ref write STORE lens.u32 sorted.raw
 *       ovStoreWriter (the sequential store build, ovStoreBuild.C's last step) over the
 *       records of sorted.raw (six uint32 words each, sorted by ovOverlap::operator<);
 *       lens.u32 holds the read lengths of IDs 1..n as uint32.
 *   ovstore_ref dump STORE lens.u32 out.raw
 *       every overlap of STORE, read back with ovStore::readOverlap over the whole read
 *       range, to out.raw in the same word layout, and read by read with
 *       ovStore::loadOverlapsForRead to out.raw.perread; prints the total of the
 *       overlaps per read that the store's index gives as "numOverlapsPerRead: <n>". */
#include "ovs_shim.H"

#include <string>

#include REF_OVOVERLAP_C
#include REF_OVSTOREFILE_C
#include REF_OVSTOREHISTOGRAM_C
#include REF_OVSTOREWRITER_C
#include REF_OVSTORE_C

bool fetchFromObjectStore(char *) { return false; }   // no object store here

static std::vector<uint32> load_lens(const char *path) {
  std::vector<uint32> len(1, 0);
  FILE *F = fopen(path, "rb");
  if (!F) fprintf(stderr, "cannot open %s\n", path), exit(1);
  uint32 v;
  while (fread(&v, 4, 1, F) == 1) len.push_back(v);
  fclose(F);
  return len;
}

int main(int argc, char **argv) {
  if (argc != 5 || (strcmp(argv[1], "write") != 0 && strcmp(argv[1], "dump") != 0)) {
    fprintf(stderr, "usage: %s write|dump STORE lens.u32 records.raw\n", argv[0]);
    return 1;
  }
  sqStore seq(load_lens(argv[3]));

  if (strcmp(argv[1], "write") == 0) {
    FILE *F = fopen(argv[4], "rb");
    if (!F) return 1;
    ovStoreWriter *w = new ovStoreWriter(argv[2], &seq);
    uint32         b[6];
    while (fread(b, 4, 6, F) == 6) {
      ovOverlap o;
      o.sqStoreAttach(&seq);
      o.a_iid      = b[0];
      o.b_iid      = b[1];
      o.dat.dat[0] = ((uint64)b[2] << 32) | b[3];
      o.dat.dat[1] = ((uint64)b[4] << 32) | b[5];
      w->writeOverlap(&o);
    }
    fclose(F);
    delete w;
    return 0;
  }

  // Every overlap, in store order: setRange over all reads, then readOverlap (as
  // ovStoreDump does, ovStoreDump.C:956); then every read's overlaps again through the
  // index with loadOverlapsForRead, into <out>.perread.
  ovStore *st = new ovStore(argv[2], &seq);
  auto     put = [](FILE *O, const ovOverlap &o) {
    uint32 v[6] = {o.a_iid, o.b_iid, (uint32)(o.dat.dat[0] >> 32), (uint32)o.dat.dat[0], (uint32)(o.dat.dat[1] >> 32),
                   (uint32)o.dat.dat[1]};
    fwrite(v, 4, 6, O);
  };
  uint32 *nopr  = st->numOverlapsPerRead();
  uint64  total = 0;
  for (uint32 i = 0; i <= seq.sqStore_lastReadID(); i++) total += nopr[i];
  delete[] nopr;
  FILE *O = fopen(argv[4], "wb");
  if (!O) return 1;
  if (total > 0) {   // on a store without overlaps readOverlap() reads past the index
    st->setRange(1, seq.sqStore_lastReadID());
    ovOverlap o;
    while (st->readOverlap(&o)) put(O, o);
  }
  fclose(O);
  std::string per = std::string(argv[4]) + ".perread";
  FILE       *P   = fopen(per.c_str(), "wb");
  if (!P) return 1;
  // A fresh reader: setRange() opens a data file without noting which one
  // (ovStore.C:360-400), so loadOverlapsForRead() after it can read the wrong file.
  delete st;
  st             = new ovStore(argv[2], &seq);
  ovOverlap *ovl = NULL;
  uint32     ovlMax = 0;
  for (uint32 id = 1; id <= seq.sqStore_lastReadID(); id++) {
    const uint32 n = st->loadOverlapsForRead(id, ovl, ovlMax);
    for (uint32 k = 0; k < n; k++) put(P, ovl[k]);
  }
  fclose(P);
  delete[] ovl;
  printf("numOverlapsPerRead: %llu\n", (unsigned long long)total);
  delete st;
  return 0;
}
