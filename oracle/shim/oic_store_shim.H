/* oic_store_shim.H -- test infrastructure only.
 *
 * The utility functions canu's src/stores/ovOverlap.C names beyond what
 * oic_ref_shim.H provides: the decimal formatter, a string-to-double parser and the
 * whitespace word splitter its display and parse routines use.  They live in the
 * meryl-utility submodule, absent from the reference tree; these are minimal
 * implementations so that ovOverlap.C (ovOverlap::swapIDs) and ovStoreFilter.C compile
 * where they lie, for the overlap-store oracle (oracle/store_ref.C).  Nothing here
 * touches the record arithmetic. */
#pragma once

#include <cstdlib>
#include <cstring>
#include <vector>

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
