// oic_synth -- seeded synthetic genomes and long reads for the overlap stage.
//
// Produces the read sets the overlap benchmarks are defined on: an iid uniform
// ACGT genome, optionally with an interspersed repeat family (N copies of one
// W bp consensus, each copy mutated at a per-copy divergence) and tandem arrays
// of one short unit; reads sampled at a target coverage with uniform starts,
// half of them reverse-complemented, lengths from a lognormal, normal or Pareto
// law, and sequencing errors split between substitutions, insertions and
// deletions in a given ratio.  Output is an oic_seqdb container
// (include/oic_seqdb.h).  Optionally writes the list of frequent k-mers (canonical
// k-mers whose multiplicity in the genome exceeds a threshold), one per line, the
// format overlapInCore's -k skip file takes.
//
// All randomness comes from one xoshiro256** stream seeded through splitmix64, so a
// seed gives the same reads on every host.

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include <algorithm>

#include "oic_seqdb.h"

namespace {

struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t z = seed;
    for (int i = 0; i < 4; i++) {
      z += 0x9e3779b97f4a7c15ULL;
      uint64_t x = z;
      x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
      x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
      s[i] = x ^ (x >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    uint64_t r = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double   uniform() { return (next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
  uint64_t below(uint64_t n) { return n ? next() % n : 0; }
  double   normal() {
    double u1 = uniform(), u2 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

const char kBases[4] = {'A', 'C', 'G', 'T'};

char randomBase(Rng &r) { return kBases[r.below(4)]; }

char otherBase(Rng &r, char b) {
  char c;
  do {
    c = randomBase(r);
  } while (c == b);
  return c;
}

char complement(char c) {
  switch (c) {
    case 'A': return 'T';
    case 'C': return 'G';
    case 'G': return 'C';
    case 'T': return 'A';
    default:  return 'N';
  }
}

// Mutate a copy of `src` with `rate` edits per base: 80% substitutions, 10% insertions,
// 10% deletions.
std::string mutateCopy(Rng &r, const std::string &src, double rate) {
  std::string out;
  out.reserve(src.size() + 16);
  for (char b : src) {
    if (r.uniform() >= rate) {
      out.push_back(b);
      continue;
    }
    double u = r.uniform();
    if (u < 0.8)
      out.push_back(otherBase(r, b));
    else if (u < 0.9) {
      out.push_back(randomBase(r));
      out.push_back(b);
    }  // else deletion
  }
  return out;
}

struct Options {
  uint64_t genome      = 5000000;
  double   coverage    = 20.0;
  std::string lenDist  = "lognormal";
  double   lenMean     = 8000, lenSd = 3000, lenMin = 1000, lenMax = 30000;
  double   paretoAlpha = 1.5;
  double   err         = 0.02;
  double   rSub = 1, rIns = 1, rDel = 1;
  double   rcFrac      = 0.5;
  uint32_t repCopies   = 0;
  uint32_t repLen      = 6000;
  double   repDiv      = 0.01;
  double   tandemFrac  = 0.0;
  uint32_t tandemUnit  = 171;
  double   tandemDiv   = 0.02;
  uint64_t seed        = 1;
  std::string out;
  std::string skipOut;
  uint32_t skipK       = 22;
  uint32_t skipMin     = 11;
  std::string genomeOut;
  double   nRate       = 0.0;   // per-base chance that a read base is reported as N
  uint32_t libs        = 1;     // library IDs drawn uniformly from 1..libs
};

void usage() {
  fprintf(stderr,
          "usage: oic_synth --out reads.seqdb [--genome N] [--coverage X]\n"
          "  [--len-dist lognormal|normal|pareto] [--len-mean M] [--len-sd S] [--len-min a] [--len-max b]\n"
          "  [--pareto-alpha A] [--err E] [--ratio sub:ins:del] [--rc-frac F]\n"
          "  [--repeat-copies N] [--repeat-len W] [--repeat-div D]\n"
          "  [--tandem-frac F] [--tandem-unit U] [--tandem-div D] [--seed S]\n"
          "  [--skip-out kmers.txt --skip-k K --skip-min-count C] [--genome-out g.txt]\n"
          "  [--n-rate P] [--libs L]\n");
  exit(1);
}

Options parse(int argc, char **argv) {
  Options o;
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i];
    auto val      = [&]() -> const char * {
      if (i + 1 >= argc) usage();
      return argv[++i];
    };
    if (a == "--genome") o.genome = strtoull(val(), NULL, 10);
    else if (a == "--coverage") o.coverage = atof(val());
    else if (a == "--len-dist") o.lenDist = val();
    else if (a == "--len-mean") o.lenMean = atof(val());
    else if (a == "--len-sd") o.lenSd = atof(val());
    else if (a == "--len-min") o.lenMin = atof(val());
    else if (a == "--len-max") o.lenMax = atof(val());
    else if (a == "--pareto-alpha") o.paretoAlpha = atof(val());
    else if (a == "--err") o.err = atof(val());
    else if (a == "--ratio") {
      if (sscanf(val(), "%lf:%lf:%lf", &o.rSub, &o.rIns, &o.rDel) != 3) usage();
    } else if (a == "--rc-frac") o.rcFrac = atof(val());
    else if (a == "--repeat-copies") o.repCopies = (uint32_t)strtoul(val(), NULL, 10);
    else if (a == "--repeat-len") o.repLen = (uint32_t)strtoul(val(), NULL, 10);
    else if (a == "--repeat-div") o.repDiv = atof(val());
    else if (a == "--tandem-frac") o.tandemFrac = atof(val());
    else if (a == "--tandem-unit") o.tandemUnit = (uint32_t)strtoul(val(), NULL, 10);
    else if (a == "--tandem-div") o.tandemDiv = atof(val());
    else if (a == "--seed") o.seed = strtoull(val(), NULL, 10);
    else if (a == "--out") o.out = val();
    else if (a == "--skip-out") o.skipOut = val();
    else if (a == "--skip-k") o.skipK = (uint32_t)strtoul(val(), NULL, 10);
    else if (a == "--skip-min-count") o.skipMin = (uint32_t)strtoul(val(), NULL, 10);
    else if (a == "--genome-out") o.genomeOut = val();
    else if (a == "--n-rate") o.nRate = atof(val());
    else if (a == "--libs") o.libs = (uint32_t)strtoul(val(), NULL, 10);
    else usage();
  }
  if (o.out.empty() && o.genomeOut.empty()) usage();
  return o;
}

// Build the genome: iid bases, then repeat copies and tandem arrays written over it.
std::string makeGenome(Rng &r, const Options &o) {
  std::string g(o.genome, 'A');
  for (uint64_t i = 0; i < o.genome; i++)
    g[i] = randomBase(r);

  if (o.repCopies > 0 && o.repLen > 0 && (uint64_t)o.repCopies * o.repLen * 2 <= o.genome) {
    std::string cons(o.repLen, 'A');
    for (auto &c : cons) c = randomBase(r);
    uint64_t slot = o.genome / o.repCopies;   // one copy per slot: copies never overlap
    for (uint32_t c = 0; c < o.repCopies; c++) {
      std::string copy = mutateCopy(r, cons, o.repDiv);
      if (r.uniform() < 0.5) {                // copies on both strands
        std::reverse(copy.begin(), copy.end());
        for (auto &b : copy) b = complement(b);
      }
      uint64_t room = slot > copy.size() ? slot - copy.size() : 0;
      uint64_t pos  = (uint64_t)c * slot + r.below(room + 1);
      for (uint64_t i = 0; i < copy.size() && pos + i < o.genome; i++)
        g[pos + i] = copy[i];
    }
  }

  if (o.tandemFrac > 0 && o.tandemUnit > 0) {
    std::string unit(o.tandemUnit, 'A');
    for (auto &c : unit) c = randomBase(r);
    uint64_t want = (uint64_t)(o.tandemFrac * (double)o.genome);
    uint64_t done = 0;
    while (done < want) {
      uint64_t arr = 10000 + r.below(20001);   // arrays of 10-30 kb
      if (arr > want - done) arr = want - done;
      if (arr < o.tandemUnit) break;
      std::string a;
      while (a.size() < arr) a += mutateCopy(r, unit, o.tandemDiv);
      a.resize(arr);
      uint64_t pos = r.below(o.genome - arr + 1);
      memcpy(&g[pos], a.data(), arr);
      done += arr;
    }
  }
  return g;
}

double sampleLength(Rng &r, const Options &o) {
  double L;
  if (o.lenDist == "lognormal") {
    double s2 = std::log(1.0 + (o.lenSd * o.lenSd) / (o.lenMean * o.lenMean));
    double mu = std::log(o.lenMean) - s2 / 2.0;
    do {
      L = std::exp(mu + std::sqrt(s2) * r.normal());
    } while (L < o.lenMin);
  } else if (o.lenDist == "normal") {
    do {
      L = o.lenMean + o.lenSd * r.normal();
    } while (L < o.lenMin);
  } else if (o.lenDist == "pareto") {
    double u = r.uniform();
    if (u < 1e-300) u = 1e-300;
    L = o.lenMin / std::pow(u, 1.0 / o.paretoAlpha);
  } else {
    fprintf(stderr, "unknown --len-dist '%s'\n", o.lenDist.c_str());
    exit(1);
  }
  if (L > o.lenMax) L = o.lenMax;
  return std::floor(L);
}

void writeSkipList(const std::string &g, const Options &o) {
  uint32_t K = o.skipK;
  if (K == 0 || K > 31 || g.size() < K) return;
  auto code = [](char c) -> int {
    switch (c) { case 'A': return 0; case 'C': return 1; case 'G': return 2; case 'T': return 3; }
    return -1;
  };
  std::vector<uint64_t> keys;
  keys.reserve(g.size());
  uint64_t mask = (K == 32) ? ~0ULL : ((1ULL << (2 * K)) - 1);
  uint64_t fw = 0, rv = 0;
  uint32_t valid = 0;
  for (size_t i = 0; i < g.size(); i++) {
    int c = code(g[i]);
    if (c < 0) { valid = 0; fw = rv = 0; continue; }
    fw = ((fw << 2) | (uint64_t)c) & mask;                          // first base most significant
    rv = (rv >> 2) | ((uint64_t)(3 - c) << (2 * (K - 1)));
    if (++valid >= K) keys.push_back(std::min(fw, rv));
  }
  std::sort(keys.begin(), keys.end());
  FILE *F = fopen(o.skipOut.c_str(), "w");
  if (!F) { perror(o.skipOut.c_str()); exit(1); }
  std::vector<char> buf(K + 1, 0);
  uint64_t n = 0;
  for (size_t i = 0; i < keys.size();) {
    size_t j = i;
    while (j < keys.size() && keys[j] == keys[i]) j++;
    if (j - i >= o.skipMin) {
      uint64_t k = keys[i];
      for (uint32_t p = 0; p < K; p++)
        buf[K - 1 - p] = kBases[(k >> (2 * p)) & 3];
      fprintf(F, "%s\n", buf.data());
      n++;
    }
    i = j;
  }
  fclose(F);
  fprintf(stderr, "oic_synth: %lu frequent %u-mers (genome multiplicity >= %u) -> %s\n",
          (unsigned long)n, K, o.skipMin, o.skipOut.c_str());
}

}  // namespace

int main(int argc, char **argv) {
  Options o = parse(argc, argv);
  Rng     r(o.seed);

  std::string g = makeGenome(r, o);
  if (!o.genomeOut.empty()) {
    FILE *F = fopen(o.genomeOut.c_str(), "w");
    if (!F) { perror(o.genomeOut.c_str()); return 1; }
    fwrite(g.data(), 1, g.size(), F);
    fclose(F);
  }
  if (!o.skipOut.empty())
    writeSkipList(g, o);
  if (o.out.empty())
    return 0;

  double pSub = o.rSub / (o.rSub + o.rIns + o.rDel);
  double pIns = o.rIns / (o.rSub + o.rIns + o.rDel);

  std::vector<uint32_t> lens, libs;
  std::string           bases;
  double                target = o.coverage * (double)o.genome;
  double                total  = 0;
  std::string           read;
  while (total < target) {
    uint64_t L = (uint64_t)sampleLength(r, o);
    if (L > o.genome) L = o.genome;
    if (L < 1) L = 1;
    uint64_t start = r.below(o.genome - L + 1);
    read.clear();
    for (uint64_t i = 0; i < L; i++) {
      char b = g[start + i];
      if (r.uniform() >= o.err) {
        read.push_back(b);
        continue;
      }
      double u = r.uniform();
      if (u < pSub)
        read.push_back(otherBase(r, b));
      else if (u < pSub + pIns) {
        read.push_back(randomBase(r));
        read.push_back(b);
      }  // else deletion
    }
    if (r.uniform() < o.rcFrac) {
      std::reverse(read.begin(), read.end());
      for (auto &b : read) b = complement(b);
    }
    if (read.empty()) continue;
    if (o.nRate > 0)
      for (auto &b : read)
        if (r.uniform() < o.nRate) b = 'N';
    libs.push_back(o.libs > 1 ? 1 + (uint32_t)r.below(o.libs) : 1);
    lens.push_back((uint32_t)read.size());
    bases += read;
    total += (double)L;
  }
  if (oic_seqdb_write(o.out.c_str(), (uint32_t)lens.size(), libs.data(), lens.data(), bases.data()) != 0) {
    fprintf(stderr, "oic_synth: failed to write '%s'\n", o.out.c_str());
    return 1;
  }
  fprintf(stderr, "oic_synth: genome %lu bp, %zu reads, %zu bases -> %s\n", (unsigned long)o.genome,
          lens.size(), bases.size(), o.out.c_str());
  return 0;
}
