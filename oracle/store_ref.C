/* store_ref.C -- test infrastructure only: the loading, filtering and sorting steps of
 * canu's ovStoreBuild run by canu's own code, as the checker of the engine's store sort.
 *
 * canu's src/stores/ovOverlap.C (ovOverlap::swapIDs, the ovOverlap record) and
 * src/stores/ovStoreFilter.C (ovStoreFilter::filterOverlap) are compiled where they lie:
 * this file includes them by path (REF_OVOVERLAP_C, REF_FILTER_C, set by
 * oracle/Makefile.store).  Their own headers' include guards are set first, so the
 * shim's stand-ins (oracle/shim) are used for the read store and the utility
 * functions, and the real ovOverlap.H for the record.
 *
 *   store_ref maxErate nReads in.raw out.raw
 *
 * in.raw holds overlap records as six uint32 words each (ovFile's full record); the
 * program keeps each record and its ID-swapped copy when any of forUTG/forOBT/forDUP is
 * set after the filter (ovStoreBuild.C:166-212), sorts them with std::sort and
 * ovOverlap::operator< (ovStoreBuild.C:255), writes them to out.raw in the same word
 * layout, and prints the filter's counters. */
#include "oic_ref_shim.H"
#include "oic_store_shim.H"

#include <algorithm>
#include <vector>

// The interface of canu's ovStoreFilter (declared in src/stores/ovStore.H, which needs
// the absent utility submodule); the member order is the reference's, so that the
// compiled ovStoreFilter.C sees the same object.
class ovStoreFilter {
public:
  ovStoreFilter(sqStore *seq_, double maxErate);
  ~ovStoreFilter();
  void   filterOverlap(ovOverlap &foverlap, ovOverlap &roverlap);
  void   resetCounters(void);
  uint64 savedUnitigging(void) { return saveUTG; }
  uint64 savedTrimming(void) { return saveOBT; }
  uint64 filteredNoTrim(void) { return skipOBT; }
  uint64 filteredErate(void) { return skipERATE; }
  uint64 filteredFlipped(void) { return skipFLIPPED; }

public:
  sqStore *seq;
  uint32   maxID;
  uint32   maxEvalue;
  uint64   saveUTG;
  uint64   saveOBT;
  uint64   skipOBT;
  uint64   skipERATE;
  uint64   skipFLIPPED;

private:
  char *skipReadOBT;
};

#define AS_OVSTORE_H
#define SQSTORE_H
#include REF_OVOVERLAP_C
#include REF_FILTER_C

int main(int argc, char **argv) {
  if (argc != 5) {
    fprintf(stderr, "usage: %s maxErate nReads in.raw out.raw\n", argv[0]);
    return 1;
  }
  const double maxErate = atof(argv[1]);
  sqStore      seq(nullptr, (uint32)strtoul(argv[2], NULL, 10));
  FILE        *F = fopen(argv[3], "rb");
  if (!F) return 1;
  std::vector<uint32> w;
  uint32              buf[6];
  while (fread(buf, 4, 6, F) == 6) w.insert(w.end(), buf, buf + 6);
  fclose(F);

  ovStoreFilter          filter(&seq, maxErate);
  std::vector<ovOverlap> ovls;
  for (size_t i = 0; i + 6 <= w.size(); i += 6) {
    ovOverlap f, r;
    f.a_iid      = w[i + 0];
    f.b_iid      = w[i + 1];
    f.dat.dat[0] = ((uint64)w[i + 2] << 32) | w[i + 3];
    f.dat.dat[1] = ((uint64)w[i + 4] << 32) | w[i + 5];
    filter.filterOverlap(f, r);
    if (f.dat.ovl.forUTG || f.dat.ovl.forOBT || f.dat.ovl.forDUP) ovls.push_back(f);
    if (r.dat.ovl.forUTG || r.dat.ovl.forOBT || r.dat.ovl.forDUP) ovls.push_back(r);
  }
  std::sort(ovls.begin(), ovls.end());

  FILE *O = fopen(argv[4], "wb");
  if (!O) return 1;
  for (const ovOverlap &o : ovls) {
    uint32 v[6] = {o.a_iid, o.b_iid, (uint32)(o.dat.dat[0] >> 32), (uint32)o.dat.dat[0], (uint32)(o.dat.dat[1] >> 32),
                   (uint32)o.dat.dat[1]};
    fwrite(v, 4, 6, O);
  }
  fclose(O);
  printf("%zu %llu %llu %llu %llu %llu\n", ovls.size(), (unsigned long long)filter.savedUnitigging(),
         (unsigned long long)filter.savedTrimming(), (unsigned long long)filter.filteredErate(),
         (unsigned long long)filter.filteredNoTrim(), (unsigned long long)filter.filteredFlipped());
  return 0;
}
