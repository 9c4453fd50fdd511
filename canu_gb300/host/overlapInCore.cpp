// overlapInCore -- drop-in command line for canu's overlap stage on one GB300.
//
// Takes the reference's command line (overlapInCore.C:283-450) and writes what it
// writes: the overlap records of ovFile(ovFileFullWrite) -- snappy-compressed blocks,
// ovStoreFile.C:212-286 -- to -o, the <prefix>.oc per-read counts (ovStoreFile.H:50-115)
// and the -s stats file (overlapInCore.C:539-560).  All overlap computation happens in
// liboic_gpu.so; the files are written by its oic_ovfile.h functions.  The output files
// are opened before any work starts, as the reference opens its ovFile
// (overlapInCore.C:169), and a failed open, write or close exits with status 1, so a
// pipeline that renames the output only after success never sees a partial file.
//
// Differences from the reference command line:
//   * the positional store argument is an oic_seqdb read container (include/oic_seqdb.h);
//   * -l <n> (a per-read overlap cap that makes read pairs depend on each other) is
//     rejected;
//   * --gpu-device <d> picks the CUDA device; --ovb-raw writes the six-word records
//     unframed instead of in snappy blocks (--ovb-snappy, the default, is accepted);
//   * --gpu-tune key=value[,key=value...] sets DP launch fields of oic_tuning
//     (narrowArena, wideMinLen, wideThreads, wideTile, wideBandW, wideCtas, wideArena,
//     forceWide, noGraph, wideMode), and --gpu-autotune <n> times the DP grid on the first n ref reads
//     against the first hash block and keeps the fastest configuration (oic_autotune).
//     Neither changes the records;
//   * --gpu-metrics <file> writes the run's counters, device times and rates as JSON
//     (oic_stats_json), a sidecar the reference does not have.
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "oic_gpu.h"
#include "oic_ovfile.h"
#include "oic_seqdb.h"

namespace {

bool isFile(const char *p) {
  struct stat st;
  return p && stat(p, &st) == 0 && S_ISREG(st.st_mode);
}

void decodeRange(const char *s, uint32_t &bgn, uint32_t &end) {
  char *e = nullptr;
  bgn     = (uint32_t)strtoul(s, &e, 10);
  end     = bgn;
  if (e && *e == '-') end = (uint32_t)strtoul(e + 1, nullptr, 10);
}

void usage(const char *prog) {
  fprintf(stderr, "USAGE:  %s [options] <seqStorePath>\n", prog);
  fprintf(stderr, "  -partial -h a-b -H a-b -r a-b -R a-b -k <int|file> -m -u -z -t <n>\n");
  fprintf(stderr, "  --hashbits n --hashdatalen n --hashload f --maxerate f --alignnoise f\n");
  fprintf(stderr, "  --minlength n --minkmers -o out.ovb -s out.stats [--gpu-device d] [--ovb-raw]\n");
  fprintf(stderr, "  [--gpu-metrics metrics.json]\n");
  fprintf(stderr, "  [--gpu-tune key=value,...] [--gpu-autotune nRefs]\n");
}

// Mark_Skip_Kmers file format (Build_Hash_Index.C:203-246): one k-mer per line (first
// whitespace-delimited token), FASTA '>' header lines skipped.
int readSkipFile(const char *path, uint32_t K, std::string &out) {
  FILE *F = fopen(path, "r");
  if (!F) {
    fprintf(stderr, "Failed to open '%s': %s\n", path, strerror(errno));
    return 1;
  }
  char line[1024];
  int  lineNum = 0;
  while (fgets(line, sizeof(line), F)) {
    lineNum++;
    if (line[0] == '>') {
      if (!fgets(line, sizeof(line), F)) break;
      lineNum++;
    }
    for (int i = 0; line[i]; i++)
      if (line[i] == ' ' || line[i] == '\t' || line[i] == '\n' || line[i] == '\r') line[i] = 0;
    size_t len = strlen(line);
    if (len != K) {
      fprintf(stderr, "Short kmer skip kmer '%s' at line %d, expecting length %u got length %zu.\n", line, lineNum, K,
              len);
      fclose(F);
      return 1;
    }
    out.append(line, K);
  }
  fclose(F);
  return 0;
}

// Opens path for writing and closes it again: the check the reference makes when it
// creates its output files, before any work.
bool canWrite(const char *path) {
  FILE *F = fopen(path, "wb");
  if (!F) {
    fprintf(stderr, "Failed to open '%s' for writing: %s\n", path, strerror(errno));
    return false;
  }
  if (fclose(F) != 0) {
    fprintf(stderr, "Failed to close '%s': %s\n", path, strerror(errno));
    return false;
  }
  return true;
}

// --gpu-tune key=value[,key=value...] into an oic_tuning.
bool parseTuning(const char *s, oic_tuning &t) {
  std::string all = s;
  size_t      p   = 0;
  while (p <= all.size()) {
    size_t      q   = all.find(',', p);
    std::string kv  = all.substr(p, q == std::string::npos ? std::string::npos : q - p);
    size_t      eq  = kv.find('=');
    if (eq == std::string::npos) return false;
    std::string k   = kv.substr(0, eq);
    uint64_t    v   = strtoull(kv.c_str() + eq + 1, nullptr, 10);
    if (k == "narrowArena") t.narrowArena = (uint32_t)v;
    else if (k == "wideMinLen") t.wideMinLen = (uint32_t)v;
    else if (k == "wideThreads") t.wideThreads = (uint32_t)v;
    else if (k == "wideTile") t.wideTile = (uint32_t)v;
    else if (k == "wideBandW") t.wideBandW = (uint32_t)v;
    else if (k == "wideCtas") t.wideCtas = (uint32_t)v;
    else if (k == "wideArena") t.wideArena = v;
    else if (k == "forceWide") t.forceWide = (uint32_t)v;
    else if (k == "noGraph") t.noGraph = (uint32_t)v;
    else if (k == "wideMode") t.wideMode = (uint32_t)v;
    else return false;
    if (q == std::string::npos) break;
    p = q + 1;
  }
  return true;
}

}  // namespace

int main(int argc, char **argv) {
  oic_params P;
  oic_default_params(&P);
  P.numThreads = 1;
  const char *store = nullptr, *outName = nullptr, *statName = nullptr, *skipFile = nullptr, *metricsName = nullptr;
  int         device = 0, err = 0;
  bool        snappy = true, haveTune = false;
  oic_tuning  tune{};
  uint32_t    autotuneRefs = 0;

  for (int a = 1; a < argc; a++) {
    const char *o   = argv[a];
    auto        nxt = [&]() -> const char * {
      if (a + 1 >= argc) { err++; return "0"; }
      return argv[++a];
    };
    if (!strcmp(o, "-partial")) P.partial = 1;
    else if (!strcmp(o, "-h")) decodeRange(nxt(), P.bgnHashID, P.endHashID);
    else if (!strcmp(o, "-H")) decodeRange(nxt(), P.minLibToHash, P.maxLibToHash);
    else if (!strcmp(o, "-r")) decodeRange(nxt(), P.bgnRefID, P.endRefID);
    else if (!strcmp(o, "-R")) decodeRange(nxt(), P.minLibToRef, P.maxLibToRef);
    else if (!strcmp(o, "-k")) {
      const char *v = nxt();
      if (isFile(v)) skipFile = v;
      else P.kmerLen = (uint32_t)strtoul(v, nullptr, 10);
    } else if (!strcmp(o, "-l")) {
      long l = strtol(nxt(), nullptr, 10);
      if (l >= 1) {
        fprintf(stderr, "-l (per-read overlap limit) is not supported by this overlapper\n");
        err++;
      }
    } else if (!strcmp(o, "-m")) P.uniqueOlapPerPair = 0;
    else if (!strcmp(o, "-u")) P.uniqueOlapPerPair = 1;
    else if (!strcmp(o, "--hashbits")) P.hashBits = (uint32_t)strtoull(nxt(), nullptr, 10);
    else if (!strcmp(o, "--hashdatalen")) P.maxHashDataLen = strtoull(nxt(), nullptr, 10);
    else if (!strcmp(o, "--hashload")) P.maxHashLoad = atof(nxt());
    else if (!strcmp(o, "-o")) outName = nxt();
    else if (!strcmp(o, "-s")) statName = nxt();
    else if (!strcmp(o, "-t")) {
      long t = strtol(nxt(), nullptr, 10);
      P.numThreads = (uint32_t)(t < 1 ? 1 : t);
    } else if (!strcmp(o, "--minlength")) P.minOlapLen = (int32_t)strtol(nxt(), nullptr, 10);
    else if (!strcmp(o, "--minkmers")) P.minKmers = 1;
    else if (!strcmp(o, "--maxerate")) P.maxErate = strtof(nxt(), nullptr);     // overlapInCore.C:380
    else if (!strcmp(o, "--alignnoise")) P.alignNoise = strtof(nxt(), nullptr);
    else if (!strcmp(o, "-z")) P.useHopelessCheck = 0;
    else if (!strcmp(o, "--gpu-device")) device = atoi(nxt());
    else if (!strcmp(o, "--gpu-metrics")) metricsName = nxt();
    else if (!strcmp(o, "--ovb-snappy")) snappy = true;
    else if (!strcmp(o, "--ovb-raw")) snappy = false;
    else if (!strcmp(o, "--gpu-tune")) {
      haveTune = true;
      if (!parseTuning(nxt(), tune)) fprintf(stderr, "bad --gpu-tune value\n"), err++;
    } else if (!strcmp(o, "--gpu-autotune")) autotuneRefs = (uint32_t)strtoul(nxt(), nullptr, 10);
    else if (!store) store = o;
    else {
      fprintf(stderr, "Unknown option '%s'\n", o);
      err++;
    }
  }
  if (P.kmerLen == 0) fprintf(stderr, "* No kmer length supplied; -k needed!\n"), err++;
  if (!outName) fprintf(stderr, "ERROR:  No output file name specified\n"), err++;
  if (err || !store) {
    usage(argv[0]);
    return 1;
  }

  char ocName[4096];
  if (oic_oc_path(outName, ocName, sizeof(ocName))) {
    fprintf(stderr, "Output name '%s' is too long\n", outName);
    return 1;
  }
  if (!canWrite(outName) || !canWrite(ocName) || (statName && !canWrite(statName)) ||
      (metricsName && !canWrite(metricsName)))
    return 1;

  // The skip list is checked before any device work too: a malformed file ends the run
  // as the reference's Mark_Skip_Kmers does.
  std::string skipKmers;
  if (skipFile && readSkipFile(skipFile, P.kmerLen, skipKmers)) return 1;

  oic_seqdb db;
  if (oic_seqdb_load(store, &db)) {
    fprintf(stderr, "Failed to load read container '%s'\n", store);
    return 1;
  }
  oic_ctx *ctx = nullptr;
  int      rc  = oic_create(&P, device, &ctx);
  if (rc) {
    fprintf(stderr, "oic_create failed (%d): %s\n", rc, ctx ? oic_last_error(ctx) : "bad parameters or no CUDA device");
    return 1;
  }
  std::vector<uint32_t> lib(db.nReads), len(db.nReads);
  std::vector<uint64_t> off(db.nReads);
  for (uint32_t i = 0; i < db.nReads; i++) {
    lib[i] = db.index[i].libID;
    len[i] = db.index[i].length;
    off[i] = db.index[i].offset;
  }
  rc = oic_set_reads(ctx, db.nReads, lib.data(), len.data(), off.data(), db.bases, db.nBases);
  if (!rc && skipFile) {
    rc = oic_set_skip_kmers(ctx, skipKmers.data(), skipKmers.size() / P.kmerLen);
    fprintf(stderr, "\nRead %zu kmers to mark to skip\n\n", skipKmers.size() / P.kmerLen);
  }
  if (!rc && haveTune) rc = oic_set_tuning(ctx, &tune);
  if (!rc && autotuneRefs) {
    // Tune on the first hash block and the first autotuneRefs ref reads of the -r range.
    uint32_t last = 0;
    rc = oic_load_hash_block(ctx, P.bgnHashID, P.endHashID, &last);
    const uint32_t r0 = P.bgnRefID < 1 ? 1 : P.bgnRefID;
    if (!rc) rc = oic_autotune(ctx, r0, r0 + autotuneRefs - 1, nullptr, 0, nullptr);
    oic_tuning best;
    if (!rc && !oic_get_tuning(ctx, &best))
      fprintf(stderr, "autotune: wideThreads %u wideTile %u wideMinLen %u\n", best.wideThreads, best.wideTile,
              best.wideMinLen);
  }
  if (!rc) rc = oic_run(ctx);
  if (rc) {
    fprintf(stderr, "overlapInCore failed (%d): %s\n", rc, oic_last_error(ctx));
    oic_destroy(ctx);
    return 1;
  }

  uint64_t n = 0;
  oic_num_overlaps(ctx, &n);
  std::vector<uint32_t> rec((size_t)n * 6);
  oic_fetch_overlaps(ctx, rec.data(), n, &n);
  oic_stats st;
  oic_get_stats(ctx, &st);
  oic_destroy(ctx);

  if (oic_ovb_write(outName, rec.data(), n, snappy ? 1 : 0)) {
    fprintf(stderr, "Failed to write '%s': %s\n", outName, strerror(errno));
    return 1;
  }
  // <prefix>.oc: u64 nOlaps, u32 oprMax, u32 opr[oprMax] (ovStoreFile.H:73-91).
  if (oic_oc_write(ocName, rec.data(), n, db.nReads)) {
    fprintf(stderr, "Failed to write '%s': %s\n", ocName, strerror(errno));
    return 1;
  }

  FILE *S = stderr;
  if (statName && !(S = fopen(statName, "w"))) {
    fprintf(stderr, "Failed to open '%s' for writing: %s\n", statName, strerror(errno));
    return 1;
  }
  int w = 0;
  w |= fprintf(S, " Kmer hits without olaps = %ld\n", (long)st.kmerHitsWithoutOlap) < 0;
  w |= fprintf(S, "    Kmer hits with olaps = %ld\n", (long)st.kmerHitsWithOlap) < 0;
  w |= fprintf(S, "  Multiple overlaps/pair = %ld\n", (long)st.multiOverlap) < 0;
  w |= fprintf(S, " Total overlaps produced = %ld\n", (long)st.totalOverlaps) < 0;
  w |= fprintf(S, "      Contained overlaps = %ld\n", (long)st.containedOverlaps) < 0;
  w |= fprintf(S, "       Dovetail overlaps = %ld\n", (long)st.dovetailOverlaps) < 0;
  w |= fprintf(S, "Rejected by short window = %ld\n", (long)st.badShortWindow) < 0;
  w |= fprintf(S, " Rejected by long window = %ld\n", (long)st.badLongWindow) < 0;
  if (S != stderr) w |= fclose(S) != 0;
  else w |= fflush(S) != 0;
  if (w) {
    fprintf(stderr, "Failed to write the stats to '%s': %s\n", statName ? statName : "stderr", strerror(errno));
    return 1;
  }

  if (metricsName) {   // the JSON sidecar: counters, device times, rates
    size_t len = 0;
    oic_stats_json(&st, nullptr, 0, &len);
    std::string js(len + 1, '\0');
    FILE *M  = fopen(metricsName, "w");
    bool  ok = M && oic_stats_json(&st, &js[0], js.size(), &len) == OIC_OK && fwrite(js.data(), 1, len, M) == len &&
              fputc('\n', M) != EOF;
    ok = (M && fclose(M) == 0) && ok;
    if (!ok) {
      fprintf(stderr, "Failed to write the metrics to '%s': %s\n", metricsName, strerror(errno));
      return 1;
    }
  }

  fprintf(stderr, "GPU: %lu overlaps; %lu seeds, %lu pairs, %lu extensions, %lu DP cells (%lu in pairs without "
                  "overlap), %lu rows; hash %.2f ms, seed %.2f ms, align %.2f ms, total %.2f ms\n",
          (unsigned long)n, (unsigned long)st.seeds, (unsigned long)st.candidatePairs, (unsigned long)st.extensions,
          (unsigned long)st.dpCells, (unsigned long)st.dpCellsNoOverlap, (unsigned long)st.dpRows, st.msHash,
          st.msSeed, st.msAlign, st.msTotal);
  fprintf(stderr, "GPU DP bins: one-warp %lu pairs %.2f ms; CTA %lu pairs (incl. reruns) %lu cells %.2f ms\n",
          (unsigned long)st.pairsNarrow, st.msNarrow, (unsigned long)st.pairsWide, (unsigned long)st.cellsWide,
          st.msWide);
  fprintf(stderr, "Bye.\n");
  oic_seqdb_free(&db);
  return 0;
}
