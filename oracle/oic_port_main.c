/*
 * oic_port_main.c -- command-line front end of the CPU oracle (test infrastructure).
 *
 * Takes overlapInCore's command line (overlapInCore.C:283-450) and writes what the
 * reference writes: the overlap records (six uint32 per record, ovStoreFile.C:262-276,
 * without snappy framing), the <prefix>.oc counts (ovStoreFile.H:73-91) and the -s
 * stats file (overlapInCore.C:550-558).  Used as the timed CPU baseline and to check
 * the CUDA path; never part of the product.
 */
#include "oic_port.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static double now(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int main(int argc, char **argv) {
  oic_port_params p;
  const char     *store, *out, *statsPath;
  if (oic_port_parse_args(argc, argv, &p, &store, &out, &statsPath)) {
    fprintf(stderr, "USAGE:  %s [options] <seqStorePath>\n", argv[0]);
    return 1;
  }
  oic_seqdb db;
  if (oic_seqdb_load(store, &db)) {
    fprintf(stderr, "failed to load '%s'\n", store);
    return 1;
  }
  oic_port_record *recs;
  uint64_t         n;
  oic_port_stats   st;
  double           t0 = now();
  int              rc = oic_port_run(&p, &db, &recs, &n, &st);
  double           t1 = now();
  if (rc) return 1;

  FILE *F = fopen(out, "wb");
  if (!F) { perror(out); return 1; }
  if (n) fwrite(recs, sizeof(oic_port_record), n, F);
  fclose(F);

  uint32_t  oprMax = db.nReads + 1;
  uint32_t *opr    = (uint32_t *)calloc(oprMax, sizeof(uint32_t));
  for (uint64_t i = 0; i < n; i++) {
    opr[recs[i].w[0]]++;
    opr[recs[i].w[1]]++;
  }
  size_t ol = strlen(out);
  char  *oc = (char *)malloc(ol + 8);
  strcpy(oc, out);
  if (ol > 4 && strcmp(oc + ol - 4, ".ovb") == 0) oc[ol - 4] = 0;
  strcat(oc, ".oc");
  FILE *C = fopen(oc, "wb");
  if (C) {
    fwrite(&n, sizeof(uint64_t), 1, C);
    fwrite(&oprMax, sizeof(uint32_t), 1, C);
    fwrite(opr, sizeof(uint32_t), oprMax, C);
    fclose(C);
  }

  FILE *S = statsPath ? fopen(statsPath, "w") : stderr;
  if (!S) S = stderr;
  fprintf(S, " Kmer hits without olaps = %ld\n", (long)st.kmerHitsWithoutOlap);
  fprintf(S, "    Kmer hits with olaps = %ld\n", (long)st.kmerHitsWithOlap);
  fprintf(S, "  Multiple overlaps/pair = %ld\n", (long)st.multiOverlap);
  fprintf(S, " Total overlaps produced = %ld\n", (long)st.totalOverlaps);
  fprintf(S, "      Contained overlaps = %ld\n", (long)st.containedOverlaps);
  fprintf(S, "       Dovetail overlaps = %ld\n", (long)st.dovetailOverlaps);
  fprintf(S, "Rejected by short window = %ld\n", (long)st.badShortWindow);
  fprintf(S, " Rejected by long window = %ld\n", (long)st.badLongWindow);
  if (S != stderr) fclose(S);
  fprintf(stderr, "oic_port: %lu overlaps, %lu seeds, %lu pairs, %lu extensions, %lu DP cells, %lu slide bases, %.3f s\n",
          (unsigned long)n, (unsigned long)st.seeds, (unsigned long)st.candidatePairs, (unsigned long)st.extensions,
          (unsigned long)st.dpCells, (unsigned long)st.slideBases, t1 - t0);
  free(recs);
  free(opr);
  free(oc);
  oic_seqdb_free(&db);
  return 0;
}
