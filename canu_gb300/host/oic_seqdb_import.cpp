// oic_seqdb_import -- reads from FASTA / FASTQ files into the read container that
// overlapInCore (this engine) reads.
//
//   oic_seqdb_import -o reads.seqdb [--min-length n] reads1.fasta [reads2.fastq ...]
//
// canu loads reads into its sqStore with sqStoreCreate, one library per input; the
// overlap stage then reads each read's ID, library, length and bases from the store.
// This tool makes the oic_seqdb container (include/oic_seqdb.h) that carries the same:
//   * read IDs 1, 2, ... in input order, files in the order given;
//   * library ID = the input file's position (1 for the first file);
//   * bases upper-cased, and every letter other than A, C, G, T turned into N (the
//     store holds ACGTN; N ends k-mers and matches anything in the alignment);
//   * reads shorter than --min-length (default 1) left out, as sqStoreCreate leaves out
//     reads below canu's minimum read length;
//   * <out>.readNames.txt: "ID<TAB>name" per kept read, the first word of its header, as
//     the sqStore's readNames.txt maps IDs to names.
// FASTA records may wrap over several lines; FASTQ records may wrap their sequence and
// quality (the quality must be as long as the sequence).  Blank lines and Windows line
// ends are accepted.  A read longer than 2^21 - 1 bases (what a read store holds) is an
// error.  Exit status 0 on success, 1 on an unreadable, malformed or unwritable file
// (nothing is written then).
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "oic_seqdb.h"

namespace {

struct Reads {
  std::vector<uint32_t>    lib, len;
  std::vector<std::string> names;
  std::string              bases;
};

// One line without its end of line ('\n', '\r\n'); false at end of file.  Reads in
// 64 KiB pieces (fgets), so long sequence lines cost one call per piece.
bool get_line(FILE *f, std::string &line) {
  line.clear();
  char buf[1 << 16];
  bool any = false;
  while (fgets(buf, sizeof(buf), f)) {
    any            = true;
    const size_t n = strlen(buf);
    if (n > 0 && buf[n - 1] == '\n') {
      line.append(buf, n - 1);
      break;
    }
    line.append(buf, n);
  }
  if (!line.empty() && line.back() == '\r') line.pop_back();
  return any;
}

bool blank(const std::string &s) {
  for (char c : s)
    if (c != ' ' && c != '\t') return false;
  return true;
}

void add_bases(std::string &out, const std::string &line) {
  for (char c : line) {
    if (c == ' ' || c == '\t') continue;
    const char u = (c >= 'a' && c <= 'z') ? (char)(c - 32) : c;
    out.push_back((u == 'A' || u == 'C' || u == 'G' || u == 'T') ? u : 'N');
  }
}

std::string first_word(const std::string &header) {
  size_t b = 1, e;
  while (b < header.size() && (header[b] == ' ' || header[b] == '\t')) b++;
  for (e = b; e < header.size() && header[e] != ' ' && header[e] != '\t'; e++) {
  }
  return header.substr(b, e - b);
}

// The longest read a store holds (AS_MAX_READLEN, 21-bit read positions).
constexpr size_t kMaxReadLen = (1u << 21) - 1;

void keep(Reads &r, uint32_t lib, const std::string &name, const std::string &seq, uint32_t minLen) {
  if (seq.size() < minLen) return;
  r.lib.push_back(lib);
  r.len.push_back((uint32_t)std::min<size_t>(seq.size(), 0xffffffffu));
  r.names.push_back(name);
  r.bases += seq;
}

// Reads one FASTA or FASTQ file; returns an error message or "".
std::string load(const char *path, uint32_t lib, uint32_t minLen, Reads &r) {
  FILE *f = fopen(path, "rb");
  if (!f) return std::string("cannot open: ") + strerror(errno);
  const size_t first = r.len.size();
  std::string line, name, seq, qual;
  bool        have = false;
  long        lineNo = 0;
  std::string err;
  while (err.empty() && get_line(f, line)) {
    lineNo++;
    if (blank(line)) continue;
    if (line[0] == '>') {   // FASTA
      if (have) keep(r, lib, name, seq, minLen);
      name = first_word(line);
      seq.clear();
      have = true;
      while (true) {
        const long at = ftell(f);
        if (!get_line(f, line)) break;
        if (!line.empty() && line[0] == '>') {
          fseek(f, at, SEEK_SET);
          break;
        }
        lineNo++;
        add_bases(seq, line);
      }
    } else if (line[0] == '@') {   // FASTQ
      if (have) keep(r, lib, name, seq, minLen);
      have = false;
      name = first_word(line);
      seq.clear();
      qual.clear();
      bool plus = false;
      while (get_line(f, line)) {
        lineNo++;
        if (!line.empty() && line[0] == '+') {
          plus = true;
          break;
        }
        add_bases(seq, line);
      }
      if (!plus) {
        err = "FASTQ record '" + name + "' has no '+' line";
        break;
      }
      while (qual.size() < seq.size() && get_line(f, line)) {
        lineNo++;
        qual += line;
      }
      if (qual.size() != seq.size()) {
        err = "FASTQ record '" + name + "': quality length " + std::to_string(qual.size()) + " differs from sequence length " +
              std::to_string(seq.size());
        break;
      }
      keep(r, lib, name, seq, minLen);
    } else {
      err = "line " + std::to_string(lineNo) + " starts neither a FASTA nor a FASTQ record";
    }
  }
  if (err.empty() && have) keep(r, lib, name, seq, minLen);
  if (err.empty() && ferror(f)) err = std::string("read error: ") + strerror(errno);
  for (size_t i = first; err.empty() && i < r.len.size(); i++)
    if (r.len[i] > kMaxReadLen)
      err = "read '" + r.names[i] + "' has " + std::to_string(r.len[i]) + " bases, more than the " +
            std::to_string(kMaxReadLen) + " a read store holds";
  fclose(f);
  return err;
}

}  // namespace

int main(int argc, char **argv) {
  const char              *out    = nullptr;
  uint32_t                 minLen = 1;
  std::vector<const char *> inputs;
  for (int a = 1; a < argc; a++) {
    if (!strcmp(argv[a], "-o") && a + 1 < argc) out = argv[++a];
    else if (!strcmp(argv[a], "--min-length") && a + 1 < argc) minLen = (uint32_t)strtoul(argv[++a], nullptr, 10);
    else if (argv[a][0] == '-') {
      fprintf(stderr, "%s: unknown option '%s'\n", argv[0], argv[a]);
      return 1;
    } else inputs.push_back(argv[a]);
  }
  if (!out || inputs.empty()) {
    fprintf(stderr, "usage: %s -o reads.seqdb [--min-length n] reads1.fasta [reads2.fastq ...]\n", argv[0]);
    return 1;
  }
  if (minLen < 1) minLen = 1;
  Reads r;
  for (size_t i = 0; i < inputs.size(); i++) {
    const std::string err = load(inputs[i], (uint32_t)(i + 1), minLen, r);
    if (!err.empty()) {
      fprintf(stderr, "%s: %s\n", inputs[i], err.c_str());
      return 1;
    }
  }
  if (r.len.size() > 0xfffffffeull) {
    fprintf(stderr, "too many reads for one container\n");
    return 1;
  }
  if (oic_seqdb_write(out, (uint32_t)r.len.size(), r.lib.data(), r.len.data(), r.bases.data())) {
    fprintf(stderr, "Failed to write '%s': %s\n", out, strerror(errno));
    return 1;
  }
  const std::string namesPath = std::string(out) + ".readNames.txt";
  FILE             *n         = fopen(namesPath.c_str(), "w");
  bool              ok        = n != nullptr;
  for (size_t i = 0; ok && i < r.names.size(); i++) ok = fprintf(n, "%zu\t%s\n", i + 1, r.names[i].c_str()) > 0;
  ok = (n && fclose(n) == 0) && ok;
  if (!ok) {
    fprintf(stderr, "Failed to write '%s': %s\n", namesPath.c_str(), strerror(errno));
    return 1;
  }
  fprintf(stderr, "%zu reads, %zu bases from %zu files into %s\n", r.len.size(), r.bases.size(), inputs.size(), out);
  return 0;
}
