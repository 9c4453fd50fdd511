/*
 * ovs_shim.H -- test infrastructure only.
 *
 * Stand-ins for the meryl-utility symbols (absent submodule in the canu tree) that
 * canu's overlap-store sources need -- src/stores/ovStore.C, ovStoreWriter.C,
 * ovStoreFile.C, ovStoreHistogram.C, ovOverlap.C -- so that those files compile where
 * they lie, into oracle/_ref/ovstore_ref, the checker of the engine's ovStore writer.
 * Also a read-length-only sqStore (canu's real sqStore.H is kept out by its include
 * guard) and the object-store fetch (no object store here).
 *
 * The file routines are the plain stdio forms of what their names say: loadFile /
 * saveFile move N objects of a type as raw bytes, writeToFile / loadFromFile the same on
 * an open FILE.  Nothing here touches overlap records or store layout.
 */
#ifndef OVS_SHIM_H
#define OVS_SHIM_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#include <assert.h>
#include <math.h>
#include <limits.h>
#include <errno.h>
#include <unistd.h>
#include <sys/stat.h>
#include <sys/types.h>
#include <algorithm>
#include <functional>
#include <vector>

/* ---------------- types.H ---------------- */

typedef uint8_t   uint8;
typedef uint16_t  uint16;
typedef uint32_t  uint32;
typedef uint64_t  uint64;
typedef int8_t    int8;
typedef int16_t   int16;
typedef int32_t   int32;
typedef int64_t   int64;

#define F_U16     "%hu"
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

/* ---------------- arrays ---------------- */

enum class _raAct : uint32 { doNothing = 0, copyData = 1, clearNew = 2 };
inline _raAct operator|(_raAct a, _raAct b) { return (_raAct)((uint32)a | (uint32)b); }
inline bool   raHas(_raAct a, _raAct b)     { return ((uint32)a & (uint32)b) != 0; }

template<typename T, typename L1, typename L2>
inline void resizeArray(T *&array, L1 arrayLen, L2 &arrayMax, uint64 newMax, _raAct act = _raAct::copyData) {
  if (array != NULL && newMax <= (uint64)arrayMax)
    return;
  T *na = new T[newMax];
  if (raHas(act, _raAct::clearNew))
    memset((void *)na, 0, sizeof(T) * newMax);
  if (array != NULL && raHas(act, _raAct::copyData) && arrayLen > 0)
    memcpy((void *)na, (void *)array, sizeof(T) * (size_t)std::min((uint64)arrayLen, newMax));
  delete[] array;
  array    = na;
  arrayMax = (L2)newMax;
}

template<typename T, typename L>
inline void allocateArray(T *&array, L &arrayMax, uint64 newMax, _raAct act = _raAct::clearNew) {
  delete[] array;
  array    = new T[newMax];
  arrayMax = (L)newMax;
  if (raHas(act, _raAct::clearNew))
    memset((void *)array, 0, sizeof(T) * newMax);
}

template<typename T, typename L>
inline void allocateArray(T *&array, L newMax, _raAct act = _raAct::clearNew) {
  delete[] array;
  array = new T[newMax];
  if (raHas(act, _raAct::clearNew))
    memset((void *)array, 0, sizeof(T) * (uint64)newMax);
}

template<typename T, typename L1, typename L2>
inline void increaseArray(T *&array, L1 arrayLen, L2 &arrayMax, uint64 increment) {
  if ((uint64)arrayLen < (uint64)arrayMax)
    return;
  resizeArray(array, arrayLen, arrayMax, (uint64)arrayMax + increment, _raAct::copyData);
}

/* ---------------- files.H ---------------- */

inline bool fileExists(const char *path) {
  struct stat st;
  return (path != NULL) && (stat(path, &st) == 0) && S_ISREG(st.st_mode);
}

inline bool directoryExists(const char *path) {
  struct stat st;
  return (path != NULL) && (stat(path, &st) == 0) && S_ISDIR(st.st_mode);
}

template<typename T>
inline void writeToFile(T &obj, const char *desc, FILE *F) {
  if (fwrite(&obj, sizeof(T), 1, F) != 1)
    fprintf(stderr, "writeToFile(%s) failed\n", desc), exit(1);
}

template<typename T>
inline void writeToFile(T *arr, const char *desc, uint64 n, FILE *F) {
  if (n > 0 && fwrite(arr, sizeof(T), n, F) != n)
    fprintf(stderr, "writeToFile(%s) failed\n", desc), exit(1);
}

template<typename T>
inline uint64 loadFromFile(T &obj, const char *desc, FILE *F, bool exact = true) {
  uint64 n = fread(&obj, sizeof(T), 1, F);
  if (exact && n != 1)
    fprintf(stderr, "loadFromFile(%s) short read\n", desc), exit(1);
  return n;
}

template<typename T>
inline uint64 loadFromFile(T *arr, const char *desc, uint64 nObj, FILE *F, bool exact = true) {
  uint64 n = nObj ? fread(arr, sizeof(T), nObj, F) : 0;
  if (exact && n != nObj)
    fprintf(stderr, "loadFromFile(%s) short read\n", desc), exit(1);
  return n;
}

enum mftType { mftReadOnly = 0 };

class memoryMappedFile {   // read into memory (the evalues file the writer never makes)
public:
  memoryMappedFile(const char *name, mftType) {
    FILE *F = fopen(name, "rb");
    if (F == NULL)
      fprintf(stderr, "memoryMappedFile: cannot open '%s'\n", name), exit(1);
    fseek(F, 0, SEEK_END);
    _data.resize((size_t)ftell(F));
    fseek(F, 0, SEEK_SET);
    if (!_data.empty() && fread(_data.data(), 1, _data.size(), F) != _data.size())
      exit(1);
    fclose(F);
  }
  void *get(uint64 off) { return _data.data() + off; }

private:
  std::vector<char> _data;
};

namespace merylutil {
inline FILE *openInputFile(const char *name) {
  FILE *F = fopen(name, "rb");
  if (F == NULL)
    fprintf(stderr, "Failed to open '%s' for reading: %s\n", name, strerror(errno)), exit(1);
  return F;
}
inline FILE *openOutputFile(const char *name) {
  FILE *F = fopen(name, "wb");
  if (F == NULL)
    fprintf(stderr, "Failed to open '%s' for writing: %s\n", name, strerror(errno)), exit(1);
  return F;
}
inline void closeFile(FILE *&F, const char * = NULL) {
  if (F != NULL && F != stdout && F != stderr && fclose(F) != 0)
    fprintf(stderr, "closeFile failed: %s\n", strerror(errno)), exit(1);
  F = NULL;
}
inline void closeFile(FILE *&F, const char *, char, const char *) { closeFile(F); }
inline off_t ftell(FILE *F) { return ::ftello(F); }
inline void  mkdir(const char *path) {
  if (::mkdir(path, 0755) != 0 && errno != EEXIST)
    fprintf(stderr, "mkdir '%s': %s\n", path, strerror(errno)), exit(1);
}
inline void unlink(const char *name) { ::unlink(name); }
inline void unlink(const char *prefix, char sep, const char *suffix) {
  char name[FILENAME_MAX + 1];
  snprintf(name, FILENAME_MAX, "%s%c%s", prefix, sep, suffix);
  ::unlink(name);
}
inline void rmdir(const char *path) { ::rmdir(path); }
inline void fseek(FILE *F, off_t off, int whence) {
  if (::fseeko(F, off, whence) != 0)
    fprintf(stderr, "fseek failed: %s\n", strerror(errno)), exit(1);
}

// The name with its last '.suffix' (after the last '/') removed.
inline void findBaseFileName(char *base, const char *name) {
  strcpy(base, name);
  char *slash = strrchr(base, '/');
  char *dot   = strrchr(base, '.');
  if (dot != NULL && (slash == NULL || dot > slash))
    *dot = 0;
}

template<typename T>
inline void loadFile(const char *name, T *obj, uint64 n) {
  FILE *F = openInputFile(name);
  loadFromFile(obj, name, n, F);
  closeFile(F);
}
template<typename T>
inline void loadFile(const char *path, char sep, const char *file, T *obj, uint64 n) {
  char name[FILENAME_MAX + 1];
  snprintf(name, FILENAME_MAX, "%s%c%s", path, sep, file);
  loadFile(name, obj, n);
}
template<typename T>
inline void saveFile(const char *name, T *obj, uint64 n) {
  FILE *F = openOutputFile(name);
  writeToFile(obj, name, n, F);
  closeFile(F);
}
template<typename T>
inline void saveFile(const char *path, char sep, const char *file, T *obj, uint64 n) {
  char name[FILENAME_MAX + 1];
  snprintf(name, FILENAME_MAX, "%s%c%s", path, sep, file);
  saveFile(name, obj, n);
}
}  // namespace merylutil

/* ---------------- strings.H (what ovOverlap.C's display / parse routines name) ---------------- */

class stringList;   // named by ovStore::addEvalues, which lives in loadErates.C (not built)

inline char *toDec(uint64 v) {
  static thread_local char buf[8][24];
  static thread_local int  k = 0;
  char *b = buf[k++ & 7];
  snprintf(b, 24, "%llu", (unsigned long long)v);
  return b;
}

inline double strtodouble(const char *s) { return strtod(s, NULL); }

class splitToWords {
public:
  splitToWords(const char *line = NULL) { split(line); }
  void split(const char *line) {
    _w.clear();
    _buf.assign(line ? line : "", line ? line + strlen(line) : NULL);
    _buf.push_back(0);
    char *p = _buf.data();
    while (*p) {
      while (*p == ' ' || *p == '\t' || *p == '\n') *p++ = 0;
      if (*p) _w.push_back(p);
      while (*p && *p != ' ' && *p != '\t' && *p != '\n') p++;
    }
  }
  uint32 numWords(void) { return (uint32)_w.size(); }
  char  *operator[](uint32 i) { return i < _w.size() ? _w[i] : (char *)""; }
  char  *operator[](int i) { return (*this)[(uint32)i]; }
  int32  toint32(uint32 i) { return (int32)strtol((*this)[i], NULL, 10); }
  uint32 touint32(uint32 i) { return (uint32)strtoul((*this)[i], NULL, 10); }
  double todouble(uint32 i) { return strtod((*this)[i], NULL); }

private:
  std::vector<char>   _buf;
  std::vector<char *> _w;
};

/* ---------------- sqStore.H (read lengths only) ---------------- */

#define SQSTORE_H
#define AS_MAX_READLEN_BITS  21
#define AS_MAX_READLEN       (((uint32)1 << AS_MAX_READLEN_BITS) - 1)

typedef uint32 sqRead_which;
const sqRead_which sqRead_unset = 0x0000;
const sqRead_which sqRead_raw   = 0x0001;
static sqRead_which sqRead_defaultVersion = sqRead_raw;

class sqStore {
public:
  explicit sqStore(const std::vector<uint32> &len) : _len(len) {}   // _len[0] unused; IDs 1..n
  uint32 sqStore_lastReadID(void) { return (uint32)_len.size() - 1; }
  uint32 sqStore_getReadLength(uint32 id, sqRead_which = sqRead_defaultVersion) {
    return id < _len.size() ? _len[id] : 0;
  }

private:
  std::vector<uint32> _len;
};

#endif
