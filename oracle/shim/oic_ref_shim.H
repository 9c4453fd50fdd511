/*
 * oic_ref_shim.H -- test infrastructure only.
 *
 * Stand-ins for the handful of meryl-utility and store symbols that canu's
 * overlapInCore sources need, so that those sources can be compiled unchanged,
 * where they lie in the canu tree, into the CPU reference binary oracle/_ref/oic_ref.
 * (canu's src/utility submodule is empty in the reference tree, so the stock
 * build cannot run.)  The reference binary is the checker for the CUDA path;
 * nothing in the product links it.
 *
 * Provided here:
 *   types.H     integer typedefs and printf format macros
 *   system.H    AS_configure, thread helpers, fileExists, resizeArray, file helpers
 *   strings.H   decodeRange, strtouint32, splitToWords (declaration only)
 *   sequence.H  reverseComplementSequence
 *   sqStore.H   sqStore / sqRead over the oic_seqdb container (include/oic_seqdb.h)
 *   sqCache.H   sqCache over the same container
 *   ovStore.H   ovFile(ovFileFullWrite): raw 6 x uint32 records + the .oc counts file
 *               (canu's ovStoreFile.C:212-286 frames the same records in snappy blocks;
 *               the raw form keeps the records byte for byte without the compression)
 */
#ifndef OIC_REF_SHIM_H
#define OIC_REF_SHIM_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#include <assert.h>
#include <math.h>
#include <limits.h>
#include <errno.h>
#include <ctype.h>
#include <cctype>
#include <cerrno>
#include <algorithm>
#include <unistd.h>
#include <sys/stat.h>
#include <omp.h>

#include "oic_seqdb.h"

/* ---------------- types.H ---------------- */

typedef uint8_t   uint8;
typedef uint16_t  uint16;
typedef uint32_t  uint32;
typedef uint64_t  uint64;
typedef int8_t    int8;
typedef int16_t   int16;
typedef int32_t   int32;
typedef int64_t   int64;

#define F_U32     "%u"
#define F_S32     "%d"
#define F_U64     "%lu"
#define F_S64     "%ld"
#define F_SIZE_T  "%zu"
#define F_U32P    "u"
#define F_S32P    "d"
#define F_U64P    "lu"
#define F_S64P    "ld"

#ifndef UNUSED
#define UNUSED(x) x __attribute__((unused))
#endif

/* ---------------- system.H ---------------- */

static inline int    AS_configure(int argc, char **argv, int = 0) { (void)argv; return argc; }
static inline uint32 getMaxThreadsAllowed(void)                   { return (uint32)omp_get_max_threads(); }

static inline uint32 setNumThreads(const char *opt) {
  int n = (int)strtol(opt, NULL, 10);
  if (n < 1)
    n = 1;
  omp_set_num_threads(n);
  return (uint32)n;
}

static inline bool fileExists(const char *path) {
  struct stat st;
  return (path != NULL) && (stat(path, &st) == 0) && S_ISREG(st.st_mode);
}

template<typename T, typename L1, typename L2>
static inline void resizeArray(T *&array, L1 arrayLen, L2 &arrayMax, uint64 newMax) {
  T *na = new T[newMax];
  if (array != NULL && arrayLen > 0)
    memcpy(na, array, sizeof(T) * (size_t)std::min((uint64)arrayLen, newMax));
  delete[] array;
  array    = na;
  arrayMax = (L2)newMax;
}

namespace merylutil {
static inline FILE *openInputFile(const char *name) {
  FILE *F = fopen(name, "r");
  if (F == NULL)
    fprintf(stderr, "Failed to open '%s' for reading: %s\n", name, strerror(errno)), exit(1);
  return F;
}
static inline void closeFile(FILE *F, const char * = NULL) {
  if (F != NULL && F != stdout && F != stderr)
    fclose(F);
}
}  // namespace merylutil

/* ---------------- strings.H ---------------- */

class splitToWords;

static inline uint32 strtouint32(const char *s) { return (uint32)strtoul(s, NULL, 10); }

static inline void decodeRange(const char *s, uint32 &bgn, uint32 &end) {
  char *e = NULL;
  bgn     = (uint32)strtoul(s, &e, 10);
  end     = bgn;
  if (e != NULL && *e == '-')
    end = (uint32)strtoul(e + 1, NULL, 10);
}

/* ---------------- sequence.H ---------------- */

static inline char oicRefComplement(char c) {
  switch (c) {
    case 'a': return 't';  case 'c': return 'g';  case 'g': return 'c';  case 't': return 'a';
    case 'A': return 'T';  case 'C': return 'G';  case 'G': return 'C';  case 'T': return 'A';
    default:  return c;
  }
}

static inline void reverseComplementSequence(char *seq, int len) {
  if (len == 0)
    len = (int)strlen(seq);
  for (int i = 0, j = len - 1; i <= j; i++, j--) {
    char a = oicRefComplement(seq[i]);
    char b = oicRefComplement(seq[j]);
    seq[i] = b;
    seq[j] = a;
  }
}

/* ---------------- sqStore.H ---------------- */

#define AS_MAX_READLEN_BITS  21
#define AS_MAX_READLEN       (((uint32)1 << AS_MAX_READLEN_BITS) - 1)

enum sqRead_which { sqRead_unset = 0, sqRead_raw = 1 };
static const sqRead_which sqRead_defaultVersion = sqRead_raw;

class sqRead {
public:
  uint32  sqRead_libraryID(void) { return _lib; }
  uint32  sqRead_length(void)    { return _len; }
  char   *sqRead_sequence(void)  { return _seq; }

  uint32  _lib = 0;
  uint32  _len = 0;
  char   *_seq = NULL;
};

class sqStore {
public:
  sqStore(const char *path) {
    if (oic_seqdb_load(path, &_db) != 0)
      fprintf(stderr, "Failed to load read container '%s'\n", path), exit(1);
  }
  // A store that only knows its read count (the overlap-store oracle, oracle/store_ref.C).
  sqStore(const char *, uint32 nReads) {
    memset(&_db, 0, sizeof(_db));
    _db.nReads = nReads;
  }
  ~sqStore() { oic_seqdb_free(&_db); }

  uint32 sqStore_lastReadID(void) { return _db.nReads; }
  uint32 sqStore_getLibraryIDForRead(uint32 id) { return _db.index[id - 1].libID; }
  uint32 sqStore_getReadLength(uint32 id, sqRead_which = sqRead_defaultVersion) {
    return _db.index[id - 1].length;
  }
  void sqStore_getRead(uint32 id, sqRead *r) {
    r->_lib = _db.index[id - 1].libID;
    r->_len = _db.index[id - 1].length;
    r->_seq = _db.bases + _db.index[id - 1].offset;
  }
  const char *bases(uint32 id) { return _db.bases + _db.index[id - 1].offset; }

  oic_seqdb _db;
};

/* ---------------- sqCache.H ---------------- */

class sqCache {
public:
  sqCache(sqStore *s) : _s(s) {}
  void   sqCache_loadReads(uint32, uint32, bool = false) {}
  uint32 sqCache_getLength(uint32 id) { return _s->sqStore_getReadLength(id); }
  bool   sqCache_getSequence(uint32 id, char *&seq, uint32 &len, uint32 &max) {
    len = _s->sqStore_getReadLength(id);
    if (seq == NULL || max < len + 1) {
      delete[] seq;
      max = len + 1;
      seq = new char[max];
    }
    memcpy(seq, _s->bases(id), len);
    seq[len] = 0;
    return true;
  }
  sqStore *_s;
};

/* ---------------- ovStore.H ---------------- */

#include "ovOverlap.H"

enum ovFileType {
  ovFileNormal            = 0,
  ovFileNormalWrite       = 1,
  ovFileFull              = 2,
  ovFileFullCounts        = 3,
  ovFileFullWrite         = 4,
  ovFileFullWriteNoCounts = 5
};

class ovFile {
public:
  ovFile(sqStore *seq, const char *name, ovFileType type) {
    (void)type;
    _F = fopen(name, "wb");
    if (_F == NULL)
      fprintf(stderr, "Failed to open '%s' for writing: %s\n", name, strerror(errno)), exit(1);
    size_t nl = strlen(name);
    _oc       = new char[nl + 8];
    strcpy(_oc, name);
    if (nl > 4 && strcmp(_oc + nl - 4, ".ovb") == 0)
      _oc[nl - 4] = 0;
    strcat(_oc, ".oc");
    _oprMax = seq->sqStore_lastReadID() + 1;
    _opr    = new uint32[_oprMax];
    memset(_opr, 0, sizeof(uint32) * _oprMax);
  }
  ~ovFile() {
    fclose(_F);
    FILE *C = fopen(_oc, "wb");
    if (C != NULL) {
      fwrite(&_nOlaps, sizeof(uint64), 1, C);
      fwrite(&_oprMax, sizeof(uint32), 1, C);
      fwrite(_opr, sizeof(uint32), _oprMax, C);
      fclose(C);
    }
    delete[] _opr;
    delete[] _oc;
  }
  void writeOverlap(ovOverlap *o) {
    uint32 w[6];
    w[0] = o->a_iid;
    w[1] = o->b_iid;
    for (uint32 ii = 0; ii < 2; ii++) {
      w[2 + 2 * ii] = (uint32)((o->dat.dat[ii] >> 32) & 0xffffffff);
      w[3 + 2 * ii] = (uint32)((o->dat.dat[ii]) & 0xffffffff);
    }
    fwrite(w, sizeof(uint32), 6, _F);
    _nOlaps++;
    _opr[o->a_iid]++;
    _opr[o->b_iid]++;
  }

  FILE   *_F      = NULL;
  char   *_oc     = NULL;
  uint64  _nOlaps = 0;
  uint32  _oprMax = 0;
  uint32 *_opr    = NULL;
};

#endif
