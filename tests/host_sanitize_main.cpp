// host_sanitize_main.cpp -- test driver: the library's host file code
// (canu_gb300/host/oic_ovfile.cpp) run under AddressSanitizer and UndefinedBehavior-
// Sanitizer by tests/test_host_sanitizers.py.  It exercises every entry point of
// include/oic_ovfile.h on valid and malformed inputs and checks the round trips; any
// sanitizer report or failed check exits non-zero.
//
//   host_sanitize_main <scratch dir>
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "oic_ovfile.h"

static int g_fail = 0;
#define CHECK(c)                                                          \
  do {                                                                    \
    if (!(c)) {                                                           \
      fprintf(stderr, "check failed at line %d: %s\n", __LINE__, #c);     \
      g_fail = 1;                                                         \
    }                                                                     \
  } while (0)

// Records with IDs in 1..maxID, A hangs inside reads of length len, random rest.
static std::vector<uint32_t> records(std::mt19937_64 &r, uint64_t n, uint32_t maxID, uint32_t len) {
  std::vector<uint32_t> w(6 * n);
  for (uint64_t i = 0; i < n; i++) {
    const uint64_t ahg5 = r() % (len / 2), ahg3 = r() % (len / 2);
    const uint64_t d0   = ahg5 | (ahg3 << 21) | ((r() & 0xffff) << 42) | ((r() & 15) << 58);
    const uint64_t d1   = r();
    uint32_t      *x    = &w[6 * i];
    x[0] = 1 + (uint32_t)(r() % maxID);
    x[1] = 1 + (uint32_t)(r() % maxID);
    x[2] = (uint32_t)(d0 >> 32);
    x[3] = (uint32_t)d0;
    x[4] = (uint32_t)(d1 >> 32);
    x[5] = (uint32_t)d1;
  }
  return w;
}

static void sort_records(std::vector<uint32_t> &w) {
  const size_t                       n = w.size() / 6;
  std::vector<std::vector<uint32_t>> v(n);
  for (size_t i = 0; i < n; i++) v[i].assign(&w[6 * i], &w[6 * i] + 6);
  std::sort(v.begin(), v.end());
  for (size_t i = 0; i < n; i++) memcpy(&w[6 * i], v[i].data(), 24);
}

static void snappy_round_trips(std::mt19937_64 &r) {
  for (size_t n : {0ul, 1ul, 3ul, 17ul, 4096ul, 65535ul, 65536ul, 65537ul, 300000ul}) {
    for (int kind = 0; kind < 3; kind++) {
      std::vector<uint8_t> src(n);
      for (size_t i = 0; i < n; i++)
        src[i] = kind == 0 ? (uint8_t)r() : kind == 1 ? (uint8_t)(i % 7) : (uint8_t)((i / 100) & 3);
      std::vector<uint8_t> comp(oic_snappy_max_length(n)), back(n + 16);
      size_t               cl = 0, bl = 0;
      CHECK(oic_snappy_compress(src.data(), n, comp.data(), &cl) == 0);
      CHECK(cl <= comp.size());
      CHECK(oic_snappy_uncompress(comp.data(), cl, back.data(), back.size(), &bl) == 0);
      CHECK(bl == n && (n == 0 || memcmp(src.data(), back.data(), n) == 0));
      // Truncated and corrupted blocks are rejected without reading or writing out of bounds.
      if (cl > 2) {
        size_t b2 = 0;
        CHECK(oic_snappy_uncompress(comp.data(), cl / 2, back.data(), back.size(), &b2) != 0 || b2 <= n);
        std::vector<uint8_t> bad(comp.begin(), comp.begin() + cl);
        for (size_t i = 1; i < bad.size(); i += 7) bad[i] ^= 0x5a;
        oic_snappy_uncompress(bad.data(), bad.size(), back.data(), back.size(), &b2);
      }
      if (n > 0) {
        size_t b3 = 0;
        CHECK(oic_snappy_uncompress(comp.data(), cl, back.data(), n - 1, &b3) != 0);   // output too small
      }
    }
  }
}

static void ovb_and_oc(std::mt19937_64 &r, const std::string &dir) {
  const uint32_t maxID = 500;
  for (uint64_t n : {0ull, 1ull, 43680ull, 43681ull, 100000ull}) {   // 43680 records = one full block
    const std::vector<uint32_t> w = records(r, n, maxID, 20000);
    for (int framing = 0; framing < 2; framing++) {
      const std::string p = dir + "/j" + std::to_string(n) + "_" + std::to_string(framing) + ".ovb";
      CHECK(oic_ovb_write(p.c_str(), w.data(), n, framing) == 0);
      if (framing) {
        uint64_t cnt = 0;
        CHECK(oic_ovb_read(p.c_str(), nullptr, 0, &cnt) == 0 && cnt == n);
        std::vector<uint32_t> back(6 * n + 6);
        CHECK(oic_ovb_read(p.c_str(), back.data(), n, &cnt) == 0 && cnt == n);
        CHECK(n == 0 || memcmp(back.data(), w.data(), 24 * n) == 0);
        if (n > 1) CHECK(oic_ovb_read(p.c_str(), back.data(), n - 1, &cnt) == 2);   // more than fits
        char oc[4096];
        CHECK(oic_oc_path(p.c_str(), oc, sizeof(oc)) == 0);
        CHECK(oic_oc_write(oc, w.data(), n, maxID) == 0);
        uint64_t              no = 0;
        uint32_t              om = 0;
        std::vector<uint32_t> opr(maxID + 1);
        CHECK(oic_oc_read(oc, &no, opr.data(), maxID, &om) == 0 && no == n && om == maxID + 1);
      }
    }
  }
  // Merge two framed jobs; the merged file holds both in order.
  const std::vector<uint32_t> a = records(r, 5000, maxID, 20000), b = records(r, 7000, maxID, 20000);
  const std::string           pa = dir + "/m1.ovb", pb = dir + "/m2.ovb", pm = dir + "/all.ovb";
  char                        oc[4096];
  CHECK(oic_ovb_write(pa.c_str(), a.data(), 5000, 1) == 0 && oic_oc_path(pa.c_str(), oc, sizeof(oc)) == 0 &&
        oic_oc_write(oc, a.data(), 5000, maxID) == 0);
  CHECK(oic_ovb_write(pb.c_str(), b.data(), 7000, 1) == 0 && oic_oc_path(pb.c_str(), oc, sizeof(oc)) == 0 &&
        oic_oc_write(oc, b.data(), 7000, maxID) == 0);
  const char *in[2] = {pa.c_str(), pb.c_str()};
  CHECK(oic_merge_outputs(pm.c_str(), in, 2) == 0);
  uint64_t              cnt = 0;
  std::vector<uint32_t> back(6 * 12000);
  CHECK(oic_ovb_read(pm.c_str(), back.data(), 12000, &cnt) == 0 && cnt == 12000);
  CHECK(memcmp(back.data(), a.data(), 24 * 5000) == 0 && memcmp(&back[6 * 5000], b.data(), 24 * 7000) == 0);
  // Malformed files and arguments.
  const std::string junk = dir + "/junk.ovb";
  FILE             *f    = fopen(junk.c_str(), "wb");
  const uint64_t    big  = 1ull << 40;
  fwrite(&big, 8, 1, f);
  fwrite("xyz", 1, 3, f);
  fclose(f);
  CHECK(oic_ovb_read(junk.c_str(), nullptr, 0, &cnt) == 2);
  CHECK(oic_ovb_read((dir + "/missing.ovb").c_str(), nullptr, 0, &cnt) == 1);
  CHECK(oic_oc_write(nullptr, a.data(), 1, maxID) == 2);
  CHECK(oic_oc_write(oc, a.data(), 5000, 3) == 2);   // IDs past the last read
}

static void ovstore(std::mt19937_64 &r, const std::string &dir) {
  const uint32_t        maxID = 300;
  std::vector<uint32_t> lens(maxID);
  for (auto &l : lens) l = 2000 + (uint32_t)(r() % 30000);
  std::vector<uint32_t> w = records(r, 20000, maxID, 2000);   // A hangs below 2000: inside every read
  sort_records(w);
  CHECK(oic_ovstore_write((dir + "/one.ovlStore").c_str(), w.data(), 20000, lens.data(), maxID, 0) == 0);
  CHECK(oic_ovstore_write((dir + "/many.ovlStore").c_str(), w.data(), 20000, lens.data(), maxID, 333) == 0);
  CHECK(oic_ovstore_write((dir + "/empty.ovlStore").c_str(), nullptr, 0, lens.data(), maxID, 0) == 0);
  std::vector<uint32_t> deep(6 * 70000);   // one read with 70000 overlaps (16-bit rank wrap)
  for (uint32_t i = 0; i < 70000; i++) {
    uint32_t *x = &deep[6 * i];
    x[0] = 7;
    x[1] = 1 + i % maxID;
    x[2] = (uint32_t)((uint64_t)(r() & 0xffff) << 10);
    x[3] = (uint32_t)(r() % 500);
    x[4] = x[5] = i;
  }
  sort_records(deep);
  CHECK(oic_ovstore_write((dir + "/deep.ovlStore").c_str(), deep.data(), 70000, lens.data(), maxID, 0) == 0);
  std::vector<uint32_t> bad = w;
  std::swap(bad[0], bad[6 * 19999]);
  CHECK(oic_ovstore_write((dir + "/bad.ovlStore").c_str(), bad.data(), 20000, lens.data(), maxID, 0) == 2);
  bad = w;
  bad[6 * 19999 + 1] = maxID + 1;
  CHECK(oic_ovstore_write((dir + "/bad2.ovlStore").c_str(), bad.data(), 20000, lens.data(), maxID, 0) == 2);
  CHECK(oic_ovstore_write((dir + "/no/such/dir").c_str(), w.data(), 20000, lens.data(), maxID, 0) == 1);
}

int main(int argc, char **argv) {
  if (argc != 2) return 2;
  std::mt19937_64 r(12345);
  snappy_round_trips(r);
  ovb_and_oc(r, argv[1]);
  ovstore(r, argv[1]);
  if (!g_fail) printf("host file code: all checks passed\n");
  return g_fail;
}
