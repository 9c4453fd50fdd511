// oic_ovfile.cpp -- the overlapper's output files as canu's ovFile writes them
// (include/oic_ovfile.h): snappy-framed .ovb blocks, the .oc per-read counts, and the
// merge of independent jobs' outputs.  Host code only.
//
// The snappy encoder and decoder are this project's own, written from the published
// snappy block format: a little-endian base-128 varint of the uncompressed length,
// then elements whose tag byte's low two bits select a literal (00: length - 1 in the
// upper six bits, or 60..63 meaning 1..4 following length bytes) or a copy of an
// earlier run of the output (01: length 4..11 and an 11-bit offset; 10: length 1..64
// and a 16-bit offset; 11: length 1..64 and a 32-bit offset).  The encoder works on
// 64 KiB fragments with a 4-byte hash of recent positions, as snappy's own does, so
// every copy stays inside its fragment and takes the 1- or 2-byte offset forms.
//
// The overlap-store directory (oic_ovstore_write) is laid out as canu's sequential store
// writer lays it out (src/stores/ovStoreWriter.C:25-130): the records' data files, the
// per-read index, the info block and the per-read overlap-score profile.
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>

#include <sys/stat.h>
#include <sys/types.h>

#include "oic_ovfile.h"

namespace {

constexpr size_t kFragment = 1u << 16;
constexpr int    kHashBits = 14;

inline uint32_t load32(const uint8_t *p) {
  uint32_t v;
  memcpy(&v, p, 4);
  return v;
}

inline uint32_t hash32(uint32_t v) { return (v * 0x1e35a7bdu) >> (32 - kHashBits); }

uint8_t *put_varint(uint8_t *d, uint64_t v) {
  while (v >= 0x80) {
    *d++ = (uint8_t)(v | 0x80);
    v >>= 7;
  }
  *d++ = (uint8_t)v;
  return d;
}

uint8_t *put_literal(uint8_t *d, const uint8_t *s, size_t n) {
  const size_t l = n - 1;
  if (l < 60) *d++ = (uint8_t)(l << 2);
  else {
    int nb = l < (1u << 8) ? 1 : l < (1u << 16) ? 2 : l < (1u << 24) ? 3 : 4;
    *d++ = (uint8_t)((59 + nb) << 2);
    for (int i = 0; i < nb; i++) *d++ = (uint8_t)(l >> (8 * i));
  }
  memcpy(d, s, n);
  return d + n;
}

// One copy element of 1..64 bytes at offset off (< 65536).
uint8_t *put_copy1(uint8_t *d, size_t off, size_t len) {
  if (len >= 4 && len <= 11 && off < 2048) {
    *d++ = (uint8_t)(1 | ((len - 4) << 2) | ((off >> 8) << 5));
    *d++ = (uint8_t)(off & 0xff);
  } else {
    *d++ = (uint8_t)(2 | ((len - 1) << 2));
    *d++ = (uint8_t)(off & 0xff);
    *d++ = (uint8_t)(off >> 8);
  }
  return d;
}

uint8_t *put_copy(uint8_t *d, size_t off, size_t len) {
  while (len >= 68) {
    d = put_copy1(d, off, 64);
    len -= 64;
  }
  if (len > 64) {   // leave at least 4 bytes for the last element
    d = put_copy1(d, off, 60);
    len -= 60;
  }
  return put_copy1(d, off, len);
}

uint8_t *compress_fragment(const uint8_t *src, size_t n, uint8_t *d, uint16_t *table) {
  memset(table, 0, sizeof(uint16_t) << kHashBits);
  size_t lit = 0, i = 0;
  if (n >= 8) {
    const size_t last = n - 4;   // a match needs 4 readable bytes
    while (i <= last) {
      const uint32_t v = load32(src + i);
      const uint32_t h = hash32(v);
      const size_t   c = table[h];
      table[h]         = (uint16_t)i;
      if (c < i && load32(src + c) == v) {
        size_t len = 4;
        while (i + len < n && src[c + len] == src[i + len]) len++;
        if (i > lit) d = put_literal(d, src + lit, i - lit);
        d = put_copy(d, i - c, len);
        for (size_t k = i + 1; k < i + len && k <= last; k++) table[hash32(load32(src + k))] = (uint16_t)k;
        i += len;
        lit = i;
      } else
        i++;
    }
  }
  if (n > lit) d = put_literal(d, src + lit, n - lit);
  return d;
}

int fail_close(FILE *f) {
  const int e = errno;
  if (f) fclose(f);
  errno = e;
  return 1;
}

bool write_all(FILE *f, const void *p, size_t n) { return n == 0 || fwrite(p, 1, n, f) == n; }

// Reads a whole file; 0 ok, 1 i/o error.
int slurp(const char *path, std::vector<uint8_t> &out) {
  FILE *f = fopen(path, "rb");
  if (!f) return 1;
  out.clear();
  uint8_t buf[1 << 16];
  size_t  k;
  while ((k = fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + k);
  if (ferror(f)) return fail_close(f);
  fclose(f);
  return 0;
}

}  // namespace

extern "C" {

size_t oic_snappy_max_length(size_t n) { return 32 + n + n / 6; }

int oic_snappy_compress(const uint8_t *src, size_t n, uint8_t *dst, size_t *dstLen) {
  if ((!src && n) || !dst || !dstLen) return 2;
  std::vector<uint16_t> table((size_t)1 << kHashBits);
  uint8_t *d = put_varint(dst, n);
  for (size_t p = 0; p < n; p += kFragment) d = compress_fragment(src + p, std::min(kFragment, n - p), d, table.data());
  *dstLen = (size_t)(d - dst);
  return 0;
}

int oic_snappy_uncompress(const uint8_t *src, size_t n, uint8_t *dst, size_t cap, size_t *dstLen) {
  if ((!src && n) || !dstLen) return 2;
  size_t   i = 0;
  uint64_t ulen = 0;
  for (int shift = 0;; shift += 7) {
    if (i >= n || shift > 63) return 2;
    const uint8_t b = src[i++];
    ulen |= (uint64_t)(b & 0x7f) << shift;
    if (!(b & 0x80)) break;
  }
  if (ulen > cap || (ulen && !dst)) return 2;
  size_t o = 0;
  while (i < n) {
    const uint8_t tag = src[i++];
    size_t len, off;
    switch (tag & 3) {
      case 0: {
        len = (size_t)(tag >> 2);
        if (len >= 60) {
          const int nb = (int)len - 59;
          if (i + nb > n) return 2;
          len = 0;
          for (int k = 0; k < nb; k++) len |= (size_t)src[i + k] << (8 * k);
          i += nb;
        }
        len += 1;
        if (i + len > n || o + len > ulen) return 2;
        memcpy(dst + o, src + i, len);
        i += len;
        o += len;
        continue;
      }
      case 1:
        if (i + 1 > n) return 2;
        len = 4 + ((tag >> 2) & 7);
        off = ((size_t)(tag >> 5) << 8) | src[i];
        i += 1;
        break;
      case 2:
        if (i + 2 > n) return 2;
        len = 1 + (tag >> 2);
        off = (size_t)src[i] | ((size_t)src[i + 1] << 8);
        i += 2;
        break;
      default:
        if (i + 4 > n) return 2;
        len = 1 + (tag >> 2);
        off = (size_t)src[i] | ((size_t)src[i + 1] << 8) | ((size_t)src[i + 2] << 16) | ((size_t)src[i + 3] << 24);
        i += 4;
        break;
    }
    if (off == 0 || off > o || o + len > ulen) return 2;
    for (size_t k = 0; k < len; k++) dst[o + k] = dst[o - off + k];   // overlapping copies repeat a pattern
    o += len;
  }
  if (o != ulen) return 2;
  *dstLen = o;
  return 0;
}

int oic_ovb_write(const char *path, const uint32_t *words, uint64_t nRecords, int framing) {
  if (!path || (!words && nRecords)) return 2;
  FILE *f = fopen(path, "wb");
  if (!f) return 1;
  const uint64_t nWords = nRecords * 6;
  if (!framing) {
    if (!write_all(f, words, nWords * 4)) return fail_close(f);
  } else {
    std::vector<uint8_t> blk(oic_snappy_max_length((size_t)OIC_OVB_BLOCK_WORDS * 4));
    for (uint64_t p = 0; p < nWords; p += OIC_OVB_BLOCK_WORDS) {
      const size_t n  = (size_t)std::min<uint64_t>(OIC_OVB_BLOCK_WORDS, nWords - p);
      size_t       bl = 0;
      oic_snappy_compress((const uint8_t *)(words + p), n * 4, blk.data(), &bl);
      const uint64_t bl64 = bl;
      if (!write_all(f, &bl64, 8) || !write_all(f, blk.data(), bl)) return fail_close(f);
    }
  }
  if (fflush(f) != 0) return fail_close(f);
  return fclose(f) != 0 ? 1 : 0;
}

int oic_ovb_read(const char *path, uint32_t *words, uint64_t maxRecords, uint64_t *nRecords) {
  if (!path || !nRecords) return 2;
  *nRecords = 0;
  std::vector<uint8_t> file;
  if (slurp(path, file)) return 1;
  std::vector<uint8_t> raw((size_t)OIC_OVB_BLOCK_WORDS * 4);
  uint64_t got = 0;
  size_t   p   = 0;
  while (p < file.size()) {
    if (p + 8 > file.size()) return 2;
    uint64_t bl;
    memcpy(&bl, file.data() + p, 8);
    p += 8;
    if (bl > file.size() - p) return 2;
    size_t n = 0;
    if (oic_snappy_uncompress(file.data() + p, (size_t)bl, raw.data(), raw.size(), &n) || n % 24) return 2;
    p += (size_t)bl;
    const uint64_t recs = n / 24;
    if (words) {
      if (got + recs > maxRecords) {
        memcpy(words + got * 6, raw.data(), (size_t)(maxRecords - got) * 24);
        *nRecords = maxRecords;
        return 2;
      }
      memcpy(words + got * 6, raw.data(), n);
    }
    got += recs;
  }
  *nRecords = got;
  return 0;
}

int oic_oc_path(const char *ovbPath, char *out, size_t cap) {
  if (!ovbPath || !out) return 2;
  std::string s     = ovbPath;
  const size_t sl   = s.rfind('/');
  const size_t dot  = s.find('.', sl == std::string::npos ? 0 : sl + 1);
  if (dot != std::string::npos) s.resize(dot);
  s += ".oc";
  if (s.size() + 1 > cap) return 2;
  memcpy(out, s.c_str(), s.size() + 1);
  return 0;
}

int oic_oc_write(const char *path, const uint32_t *words, uint64_t nRecords, uint32_t lastID) {
  if (!path || (!words && nRecords)) return 2;
  const uint32_t        oprMax = lastID + 1;
  std::vector<uint32_t> opr(oprMax, 0);
  for (uint64_t i = 0; i < nRecords; i++) {
    const uint32_t a = words[6 * i], b = words[6 * i + 1];
    if (a >= oprMax || b >= oprMax) return 2;
    opr[a]++;
    opr[b]++;
  }
  FILE *f = fopen(path, "wb");
  if (!f) return 1;
  if (!write_all(f, &nRecords, 8) || !write_all(f, &oprMax, 4) || !write_all(f, opr.data(), (size_t)oprMax * 4))
    return fail_close(f);
  if (fflush(f) != 0) return fail_close(f);
  return fclose(f) != 0 ? 1 : 0;
}

int oic_oc_read(const char *path, uint64_t *nOlaps, uint32_t *opr, uint32_t maxReads, uint32_t *oprMax) {
  if (!path || !nOlaps || !oprMax) return 2;
  std::vector<uint8_t> file;
  if (slurp(path, file)) return 1;
  if (file.size() < 12) return 2;
  memcpy(nOlaps, file.data(), 8);
  memcpy(oprMax, file.data() + 8, 4);
  if (file.size() != 12 + (size_t)*oprMax * 4) return 2;
  if (opr) {
    const uint32_t n = std::min<uint32_t>(*oprMax, maxReads + 1);
    memcpy(opr, file.data() + 12, (size_t)n * 4);
  }
  return 0;
}

int oic_merge_outputs(const char *outOvb, const char *const *inputs, uint32_t n) {
  if (!outOvb || (!inputs && n)) return 2;
  uint64_t              total = 0;
  std::vector<uint32_t> opr;
  std::vector<uint8_t>  file;
  char                  oc[4096];
  FILE *f = fopen(outOvb, "wb");
  if (!f) return 1;
  for (uint32_t k = 0; k < n; k++) {
    // The .ovb: whole blocks, checked to be framed before they are copied.
    if (slurp(inputs[k], file)) return fail_close(f);
    size_t p = 0;
    while (p < file.size()) {
      uint64_t bl;
      if (p + 8 > file.size()) { fclose(f); return 2; }
      memcpy(&bl, file.data() + p, 8);
      if (bl > file.size() - p - 8) { fclose(f); return 2; }
      p += 8 + (size_t)bl;
    }
    if (!write_all(f, file.data(), file.size())) return fail_close(f);
    // The .oc: counts summed read by read.
    if (oic_oc_path(inputs[k], oc, sizeof(oc)) || slurp(oc, file)) return fail_close(f);
    uint64_t nO;
    uint32_t om;
    if (file.size() < 12) { fclose(f); return 2; }
    memcpy(&nO, file.data(), 8);
    memcpy(&om, file.data() + 8, 4);
    if (file.size() != 12 + (size_t)om * 4) { fclose(f); return 2; }
    if (om > opr.size()) opr.resize(om, 0);
    const uint32_t *c = (const uint32_t *)(file.data() + 12);
    for (uint32_t i = 0; i < om; i++) opr[i] += c[i];
    total += nO;
  }
  if (fflush(f) != 0) return fail_close(f);
  if (fclose(f) != 0) return 1;
  if (oic_oc_path(outOvb, oc, sizeof(oc))) return 2;
  FILE *g = fopen(oc, "wb");
  if (!g) return 1;
  const uint32_t om = (uint32_t)opr.size();
  if (!write_all(g, &total, 8) || !write_all(g, &om, 4) || !write_all(g, opr.data(), opr.size() * 4))
    return fail_close(g);
  if (fflush(g) != 0) return fail_close(g);
  return fclose(g) != 0 ? 1 : 0;
}

namespace {

// One read's entry of the store's statistics file (oSH_ovlSco, ovStoreHistogram.H:41-44).
constexpr int kScorePoints = 16;
struct ScoreProfile {
  uint16_t points[kScorePoints];
  uint16_t scores[kScorePoints];
};
static_assert(sizeof(ScoreProfile) == 64, "score profile layout");

// The score profile of one read from its overlaps' scores (ovStoreHistogram.C:226-259):
// the scores sorted decreasing and sampled at up to 15 ranks spaced n/16 apart (at
// least 1, at most 10), rounded to the nearest rank; the remaining points take the last
// rank.  Ranks are stored in 16 bits, as the reference stores them.
ScoreProfile score_profile(std::vector<uint16_t> &sc) {
  std::sort(sc.begin(), sc.end(), [](uint16_t x, uint16_t y) { return x > y; });
  const uint32_t n = (uint32_t)sc.size();
  ScoreProfile   p;
  double         step = (double)n / kScorePoints;
  if (step < 1) step = 1;
  if (step > 10) step = 10;
  for (int i = 0; i < kScorePoints; i++) p.points[i] = (uint16_t)(n - 1);
  double point = 0;
  for (int i = 0; i < kScorePoints - 1 && point < n; i++, point += step) p.points[i] = (uint16_t)std::floor(point + 0.5);
  for (int i = 0; i < kScorePoints; i++) p.scores[i] = sc[p.points[i]];
  return p;
}

// Writes n objects to dir/name; 0 ok, 1 i/o failure.
int save_file(const std::string &path, const void *p, size_t bytes) {
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) return 1;
  if (!write_all(f, p, bytes)) return fail_close(f);
  if (fflush(f) != 0) return fail_close(f);
  return fclose(f) != 0 ? 1 : 0;
}

}  // namespace

int oic_ovstore_write(const char *dir, const uint32_t *rec, uint64_t nRecords, const uint32_t *readLen,
                      uint32_t maxID, uint64_t maxPerFile) {
  if (!dir || (!rec && nRecords) || (!readLen && maxID)) return 2;
  if (maxPerFile == 0) maxPerFile = OIC_OVSTORE_MAX_PER_FILE;
  if (maxPerFile > 0x7fffffffull) return 2;   // offsets in a data file are 32-bit in the index

  // The records must be a store's: IDs within 1..maxID, in (a_iid, b_iid, data) order,
  // with A hangs inside the A read (the score divides by the read's length).
  for (uint64_t i = 0; i < nRecords; i++) {
    const uint32_t *r = rec + 6 * i;
    if (r[0] == 0 || r[0] > maxID || r[1] == 0 || r[1] > maxID) return 2;
    if (i > 0 && std::lexicographical_compare(r, r + 6, r - 6, r)) return 2;
    const uint64_t d0 = ((uint64_t)r[2] << 32) | r[3];
    const uint32_t ahg5 = (uint32_t)(d0 & 0x1fffff), ahg3 = (uint32_t)((d0 >> 21) & 0x1fffff);
    if ((uint64_t)ahg5 + ahg3 > readLen[r[0] - 1]) return 2;
  }

  if (mkdir(dir, 0755) != 0 && errno != EEXIST) return 1;
  const std::string base(dir);

  // ovStoreOfft (ovStore.H:140-170): slice, file, offset in the file, records, then
  // the index of the read's first record in the store; 4 zero bytes of padding.
  struct Offt {
    uint16_t slice, piece;
    uint32_t offset, numOlaps, pad;
    uint64_t overlapID;
  };
  static_assert(sizeof(Offt) == 24, "index entry layout");
  std::vector<Offt>         index((size_t)maxID + 1);
  std::vector<ScoreProfile> prof((size_t)maxID + 1);
  memset(index.data(), 0, index.size() * sizeof(Offt));
  memset(prof.data(), 0, prof.size() * sizeof(ScoreProfile));

  // The data files (ovFile(ovFileNormalWrite), ovStoreFile.C:212-238 with _isNormal):
  // five words per record, no a_iid.  A new file starts at a read's first record once
  // the current file holds more than maxPerFile records (ovStoreWriter.C:84-101).
  uint32_t              piece = 0, bgnID = UINT32_MAX, endID = 0;
  uint64_t              inPiece = 0;
  FILE                 *f = nullptr;
  std::vector<uint16_t> scores;
  char                  name[32];
  for (uint64_t i = 0; i < nRecords; i++) {
    const uint32_t *r = rec + 6 * i;
    const uint32_t  a = r[0];
    if (f && inPiece > maxPerFile && endID < a) {
      if (fflush(f) != 0) return fail_close(f);
      if (fclose(f) != 0) return 1;
      f = nullptr;
    }
    if (!f) {
      snprintf(name, sizeof(name), "/%04u-%03u", 1u, ++piece);
      f = fopen((base + name).c_str(), "wb");
      if (!f) return 1;
      inPiece = 0;
    }
    Offt &x = index[a];
    if (inPiece > 0xffffffffull || x.numOlaps == 0xffffffffu) {   // past the index's 32-bit fields
      fclose(f);
      return 2;
    }
    if (x.numOlaps == 0) {
      x.slice     = 1;
      x.piece     = (uint16_t)piece;
      x.offset    = (uint32_t)inPiece;
      x.overlapID = i;
    }
    x.numOlaps++;
    bgnID = std::min(bgnID, a);
    endID = std::max(endID, a);
    if (!write_all(f, r + 1, 5 * sizeof(uint32_t))) return fail_close(f);
    inPiece++;

    // The record's overlap score (ovOverlap::overlapScore, ovOverlap.H:243-247):
    // 16384 x identity x (aligned A bases / A length), identity = 1 - evalue / 1e5.
    const uint64_t d0  = ((uint64_t)r[2] << 32) | r[3];
    const uint32_t ev  = (uint32_t)((d0 >> 42) & 0xffff);
    const uint32_t len = readLen[a - 1];
    const uint32_t al  = len - (uint32_t)(d0 & 0x1fffff) - (uint32_t)((d0 >> 21) & 0x1fffff);
    scores.push_back((uint16_t)std::floor(16384.0 * (1 - ev / 100000.0) * al / len));
    if (i + 1 == nRecords || rec[6 * (i + 1)] != a) {
      prof[a] = score_profile(scores);
      scores.clear();
    }
  }
  if (f) {
    if (fflush(f) != 0) return fail_close(f);
    if (fclose(f) != 0) return 1;
  }

  if (save_file(base + "/index", index.data(), index.size() * sizeof(Offt))) return 1;

  // statistics (ovStoreHistogram::saveHistogram, ovStoreHistogram.C:135-168): maxID,
  // first and last ID of the profile array (0 and maxID), the profiles.  No file when
  // the store holds no overlap.
  if (nRecords) {
    std::vector<uint8_t> st(12 + prof.size() * sizeof(ScoreProfile));
    const uint32_t       hdr[3] = {maxID, 0, maxID};
    memcpy(st.data(), hdr, 12);
    memcpy(st.data() + 12, prof.data(), prof.size() * sizeof(ScoreProfile));
    if (save_file(base + "/statistics", st.data(), st.size())) return 1;
  }

  // info (ovStoreInfo, ovStore.H:39-137): magic "canu:OVS", version 4, read-length bits,
  // first and last read ID with overlaps, maxID, records.
  struct Info {
    uint64_t magic, version;
    uint32_t readLenBits, bgnID, endID, maxID;
    uint64_t numOlaps;
  };
  static_assert(sizeof(Info) == 40, "info layout");
  const Info info = {0x53564f3a756e6163ull, 4, 21, bgnID, endID, maxID, nRecords};
  return save_file(base + "/info", &info, sizeof(info));
}

}  // extern "C"
