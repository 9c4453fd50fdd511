/*
 * oic_port.c -- CPU restatement of canu's overlapInCore hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle that tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py use to check and to time against.  The CUDA product
 * never links or calls this file.
 *
 * Each function states which reference function it restates (paths are relative to
 * canu's src/).  Parity is pinned against canu's own sources compiled with a shim
 * (oracle/Makefile.ref): identical sorted record sets, .oc counts and stats counters
 * on the fixtures in tests/golden/.
 *
 * Data layout differs from the reference where the results cannot depend on it: the
 * k-mer index is an exact key -> occurrence-list map (the reference's 21-entry
 * buckets, check bytes and probe sequence only filter and never change which
 * occurrences a k-mer has), and candidate read pairs are kept in a per-read map
 * instead of the 256-slot String_Olap table (pairs are processed independently under
 * the default -l).  Everything that can change an emitted record -- the order seeds
 * reach a pair, the match-node list rules, the DP, the traceback, the double
 * precision branch-point test -- follows the reference step for step.
 */
#define _GNU_SOURCE
#include "oic_port.h"

#include <assert.h>
#include <ctype.h>
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define AS_MAX_READLEN_BITS 21
#define AS_MAX_READLEN      ((1u << AS_MAX_READLEN_BITS) - 1)

/* overlapInCore.H:78,107,120,146 */
#define HOPELESS_MATCH      90
#define MAX_DISTINCT_OLAPS  3
#define MIN_INTERSECTION    10
#define SHIFT_SLACK         1
#define ENTRIES_PER_BUCKET  21

/* prefixEditDistance.H:35-40 */
enum { OLAP_NONE = 0, OLAP_LEFT_BRANCH_PT = 1, OLAP_RIGHT_BRANCH_PT = 2, OLAP_DOVETAIL = 3 };

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

static void *xmalloc(size_t n) {
  void *p = malloc(n ? n : 1);
  if (!p) {
    fprintf(stderr, "oic_port: out of memory (%zu bytes)\n", n);
    exit(1);
  }
  return p;
}
static void *xcalloc(size_t n, size_t s) {
  void *p = calloc(n ? n : 1, s ? s : 1);
  if (!p) {
    fprintf(stderr, "oic_port: out of memory\n");
    exit(1);
  }
  return p;
}
static void *xrealloc(void *p, size_t n) {
  p = realloc(p, n ? n : 1);
  if (!p) {
    fprintf(stderr, "oic_port: out of memory\n");
    exit(1);
  }
  return p;
}

/* ------------------------------------------------------------------------------ */
/* Parameters: overlapInCore.H:374-411 (defaults), overlapInCore.C:293-411 (parse). */

void oic_port_default_params(oic_port_params *p) {
  memset(p, 0, sizeof(*p));
  p->maxErate          = 0.06;
  p->alignNoise        = 1.0;
  p->bgnHashID         = 1;
  p->endHashID         = UINT32_MAX;
  p->maxLibToHash      = UINT32_MAX;
  p->bgnRefID          = 1;
  p->endRefID          = UINT32_MAX;
  p->maxLibToRef       = UINT32_MAX;
  p->uniqueOlapPerPair = 1;
  p->hashBits          = 22;
  p->maxHashLoad       = 0.6;
  p->maxHashDataLen    = 100000000;
  p->numThreads        = 1;
  p->useHopelessCheck  = 1;
}

static void parse_range(const char *s, uint32_t *bgn, uint32_t *end) {
  char *e = NULL;
  *bgn    = (uint32_t)strtoul(s, &e, 10);
  *end    = *bgn;
  if (e && *e == '-')
    *end = (uint32_t)strtoul(e + 1, NULL, 10);
}

static int is_regular_file(const char *path) {
  struct stat st;
  return path && stat(path, &st) == 0 && S_ISREG(st.st_mode);
}

int oic_port_parse_args(int argc, char **argv, oic_port_params *p, const char **storePath,
                        const char **outPath, const char **statsPath) {
  int err = 0;
  oic_port_default_params(p);
  *storePath = *outPath = *statsPath = NULL;
  for (int a = 1; a < argc; a++) {
    const char *o   = argv[a];
    int         has = (a + 1 < argc);
#define NEXT (has ? argv[++a] : (err++, "0"))
    if (!strcmp(o, "-partial")) p->partial = 1;
    else if (!strcmp(o, "-h")) parse_range(NEXT, &p->bgnHashID, &p->endHashID);
    else if (!strcmp(o, "-H")) parse_range(NEXT, &p->minLibToHash, &p->maxLibToHash);
    else if (!strcmp(o, "-r")) parse_range(NEXT, &p->bgnRefID, &p->endRefID);
    else if (!strcmp(o, "-R")) parse_range(NEXT, &p->minLibToRef, &p->maxLibToRef);
    else if (!strcmp(o, "-k")) {
      const char *v = NEXT;
      if (is_regular_file(v)) p->kmerSkipFile = v;
      else p->kmerLen = (uint32_t)strtoul(v, NULL, 10);
    } else if (!strcmp(o, "-l")) {
      long l = strtol(NEXT, NULL, 10);
      if (l >= 1) {
        fprintf(stderr, "oic_port: -l (per-read overlap limit) is not supported\n");
        err++;
      }
    } else if (!strcmp(o, "-m")) p->uniqueOlapPerPair = 0;
    else if (!strcmp(o, "-u")) p->uniqueOlapPerPair = 1;
    else if (!strcmp(o, "--hashbits")) p->hashBits = (uint32_t)strtoull(NEXT, NULL, 10);
    else if (!strcmp(o, "--hashdatalen")) p->maxHashDataLen = strtoull(NEXT, NULL, 10);
    else if (!strcmp(o, "--hashload")) p->maxHashLoad = atof(NEXT);
    else if (!strcmp(o, "-o")) *outPath = NEXT;
    else if (!strcmp(o, "-s")) *statsPath = NEXT;
    else if (!strcmp(o, "-t")) {
      long t = strtol(NEXT, NULL, 10);
      p->numThreads = (uint32_t)(t < 1 ? 1 : t);
    } else if (!strcmp(o, "--minlength")) p->minOlapLen = (int32_t)strtol(NEXT, NULL, 10);
    else if (!strcmp(o, "--minkmers")) p->minKmers = 1;
    else if (!strcmp(o, "--maxerate")) p->maxErate = strtof(NEXT, NULL);
    else if (!strcmp(o, "--alignnoise")) p->alignNoise = strtof(NEXT, NULL);
    else if (!strcmp(o, "-z")) p->useHopelessCheck = 0;
    else if (*storePath == NULL) *storePath = o;
    else {
      fprintf(stderr, "Unknown option '%s'\n", o);
      err++;
    }
#undef NEXT
  }
  if (p->maxErate > 0.06)
    p->useHopelessCheck = 0;
  if (p->kmerLen == 0) fprintf(stderr, "* No kmer length supplied; -k needed!\n"), err++;
  if (*outPath == NULL) fprintf(stderr, "ERROR:  No output file name specified\n"), err++;
  if (*storePath == NULL) err++;
  return err;
}

/* ------------------------------------------------------------------------------ */
/* Edit_Match_Limit: Binomial_Bound.C:36-97 (Binomial_Bound), :104-195
 * (Initialize_Match_Limit, AS_MAX_READLEN_BITS == 21 slope).                      */

static int binomial_bound(int e, double p, int start) {
  double q = 1.0 - p;
  if (start < e)
    start = e;
  for (int n = start; n < (int)AS_MAX_READLEN; n++) {
    if (n <= 35) {
      double sum = 0.0, pp = 1.0, qp = pow(q, n);
      int    coeff = 1, ct = 0, k;
      for (k = 0; k < e && 1.0 - sum > 1e-4; k++) {
        double x = coeff * pp * qp;
        sum += x;
        /* Binomial_Bound.C:63's int product overflows for n near 35 at high error
           counts and the reference's table depends on the 32-bit wraparound; the same
           wraparound as a defined unsigned product. */
        coeff = (int)((uint32_t)coeff * (uint32_t)(n - ct));
        coeff /= ++ct;
        pp *= p;
        qp /= q;
      }
      if (1.0 - sum > 1e-4)
        return n;
    } else {
      double z = (e - 0.5 - n * p) / sqrt(n * p * q);
      if (z <= 3.62)
        return n;
      double sum = 0.0, mu = 1.0, fact = 1.0, pc = exp(-n * p);
      for (int k = 0; k < e; k++) {
        sum += mu * pc / fact;
        mu *= n * p;
        fact *= k + 1;
      }
      if (1.0 - sum > 1e-4)
        return n;
    }
  }
  return (int)AS_MAX_READLEN;
}

void oic_port_match_limit(int32_t *ml, double maxErate, int32_t maxErrors) {
  int32_t e = 0, s = 1, l = imin(maxErrors, 2000);
  while (e <= 1)
    ml[e++] = 0;
  while (e < l) {
    s     = binomial_bound(e - 1, maxErate, s);
    ml[e] = s - 1;
    e++;
  }
  double sl = 0.982064188397525 / maxErate + 0.067835741959926;
  double vl = ml[e - 1] + sl;
  while (e < maxErrors) {
    ml[e] = (int32_t)ceil(vl);
    vl += sl;
    e++;
  }
}

int32_t oic_port_max_errors(double maxErate) { return 1 + (int32_t)ceil(maxErate * AS_MAX_READLEN); }

/* ------------------------------------------------------------------------------ */
/* The aligner: prefixEditDistance (prefixEditDistance.C, -forward.C, -reverse.C,
 * -extend.C).  Row e of the furthest-reaching table holds diagonals -e-2..e+2.     */

struct oic_port_aligner {
  double   maxErate;
  int      partial;
  int32_t  maxErrors;
  double   minBranchTailSlope;     /* prefixEditDistance.C:29 */
  double   branchMatchValue;       /* prefixEditDistance.C:86 */
  int32_t *matchLimit;             /* Edit_Match_Limit        */
  int32_t *errorBound;             /* Error_Bound[0..AS_MAX_READLEN] */
  int32_t **row;                   /* row[e] points at diagonal 0 of row e */
  int32_t  rowsAlloc;
  int32_t *leftDelta, *rightDelta, *stack;
  int32_t  leftDeltaLen, rightDeltaLen;
  uint64_t cells, slides;
};

oic_port_aligner *oic_port_aligner_new(double maxErate, double alignNoise, int partial) {
  oic_port_aligner *a   = (oic_port_aligner *)xcalloc(1, sizeof(*a));
  a->maxErate           = maxErate;
  a->partial            = partial;
  a->maxErrors          = oic_port_max_errors(maxErate);
  a->minBranchTailSlope = (maxErate > 0.06) ? 1.0 : 0.20;
  a->branchMatchValue   = maxErate / (1 + maxErate);
  a->matchLimit         = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(a->maxErrors + 1));
  oic_port_match_limit(a->matchLimit, maxErate * alignNoise, a->maxErrors);
  a->errorBound = (int32_t *)xmalloc(sizeof(int32_t) * (AS_MAX_READLEN + 1));
  for (uint32_t i = 0; i <= AS_MAX_READLEN; i++)
    a->errorBound[i] = (int32_t)ceil(i * maxErate);
  a->row        = (int32_t **)xcalloc((size_t)a->maxErrors + 1, sizeof(int32_t *));
  a->leftDelta  = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)a->maxErrors);
  a->rightDelta = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)a->maxErrors);
  a->stack      = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)a->maxErrors);
  return a;
}

void oic_port_aligner_free(oic_port_aligner *a) {
  if (!a) return;
  for (int32_t e = 0; e < a->rowsAlloc; e++)
    free(a->row[e] - (e + 2));
  free(a->row);
  free(a->matchLimit);
  free(a->errorBound);
  free(a->leftDelta);
  free(a->rightDelta);
  free(a->stack);
  free(a);
}

static int32_t *edit_row(oic_port_aligner *a, int32_t e) {
  while (a->rowsAlloc <= e) {
    int32_t r   = a->rowsAlloc++;
    int32_t *b  = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(2 * r + 5));
    a->row[r]   = b + r + 2;
  }
  return a->row[e];
}

/* pruneAlign, original method (prefixEditDistance.H:249-258). */
static int prune(const oic_port_aligner *a, int32_t e, int32_t v, int32_t extra) {
  return v + extra < a->matchLimit[e];
}

/* Shared traceback of Set_Right_Delta (prefixEditDistance-forward.C:32-71) and
 * Set_Left_Delta (-reverse.C:36-93): walks rows e..1 from diagonal d, pushing one
 * entry per indel; returns the value `last` reached at row 0. */
static int32_t trace_indels(oic_port_aligner *a, int32_t e, int32_t d, int32_t *out, int32_t *outLen) {
  int32_t last = a->row[e][d];
  int32_t n    = 0;
  for (int32_t k = e; k > 0; k--) {
    int32_t *p    = a->row[k - 1];
    int32_t  from = d, mx = 1 + p[d], j;
    if ((j = p[d - 1]) > mx) { from = d - 1; mx = j; }
    if ((j = 1 + p[d + 1]) > mx) { from = d + 1; mx = j; }
    if (from == d - 1) {
      out[n++] = mx - last - 1;
      d--;
      last = p[from];
    } else if (from == d + 1) {
      out[n++] = last - (mx - 1);
      d++;
      last = p[from];
    }
  }
  *outLen = n;
  return last;
}

static int sign(int32_t v) { return (v > 0) - (v < 0); }

/* Set_Right_Delta (prefixEditDistance-forward.C:32-71). */
static void set_right_delta(oic_port_aligner *a, int32_t e, int32_t d) {
  int32_t n, last = trace_indels(a, e, d, a->stack, &n);
  a->stack[n++] = last + 1;
  int32_t k = 0;
  for (int32_t i = n - 1; i > 0; i--)
    a->rightDelta[k++] = abs(a->stack[i]) * sign(a->stack[i - 1]);
  a->rightDeltaLen = n - 1;
}

/* Set_Left_Delta (prefixEditDistance-reverse.C:36-93). */
static void set_left_delta(oic_port_aligner *a, int32_t e, int32_t d, int32_t *leftover, int32_t *tEnd,
                           int32_t tLen) {
  int32_t n;
  *leftover        = trace_indels(a, e, d, a->leftDelta, &n);
  a->leftDeltaLen  = n;
  if (n > 1 && a->leftDelta[0] == 1 && *tEnd + tLen > 0) {
    a->leftDelta[0] = (a->leftDelta[1] > 0) ? a->leftDelta[1] + 1 : a->leftDelta[1] - 1;
    for (int32_t i = 2; i < n; i++)
      a->leftDelta[i - 1] = a->leftDelta[i];
    a->leftDeltaLen--;
    (*tEnd)--;
    if (a->leftDeltaLen == 0)
      (*leftover)++;
  }
}

static inline int same(char x, char y) { return x == y || x == 'n' || y == 'n'; }

/* forward (prefixEditDistance-forward.C:94-314) when step == +1 and reverse
 * (prefixEditDistance-reverse.C:114-330) when step == -1: A[step*i] is compared with
 * T[step*(i+d)].  Returns the errors; sets *aEnd and *tEnd (signed like the reference),
 * *leftover (reverse only) and *toEnd. */
static int32_t prefix_dp(oic_port_aligner *a, int step, const char *A, int32_t m, const char *T, int32_t n,
                         int32_t errorLimit, int32_t *aEnd, int32_t *tEnd, int32_t *leftover, int *toEnd) {
  const double BMV = a->branchMatchValue;
  int32_t      msLen = 0, msD = 0, msE = 0, bestD = 0, bestE = 0, longest = 0, r, e, d;
  double       maxScore = 0.0;

  (void)bestE;
  if (step > 0) a->rightDeltaLen = 0;
  else a->leftDeltaLen = 0;

  for (r = 0; r < m && same(A[step * r], T[step * r]); r++)
    ;
  a->slides += (uint64_t)r;
  edit_row(a, 0)[0] = r;

  if (r == m) {
    *aEnd = *tEnd = step * m;
    if (step < 0) *leftover = m;
    *toEnd = 1;
    return 0;
  }

  int32_t left = 0, right = 0;
  for (e = 1; e <= errorLimit; e++) {
    int32_t *cur  = edit_row(a, e);
    int32_t *prev = a->row[e - 1];
    left          = imax(left - 1, -e);
    right         = imin(right + 1, e);
    prev[left] = prev[left - 1] = prev[right] = prev[right + 1] = -2;

    for (d = left; d <= right; d++) {
      int32_t row = 1 + prev[d], j;
      if ((j = prev[d - 1]) > row) row = j;
      if ((j = 1 + prev[d + 1]) > row) row = j;
      int32_t r0 = row;
      while (row < m && row + d < n && same(A[step * row], T[step * (row + d)]))
        row++;
      a->slides += (uint64_t)(row - r0);
      a->cells++;
      cur[d] = row;

      if (row == m || row + d == n) {
        double  score   = row * BMV - e;
        int32_t tailLen = row - msLen;
        int     abort_  = 0;
        double  slope   = (double)(maxScore - score) / tailLen;
        if (a->partial && score < maxScore) abort_ = 1;
        if (e > 20 / 2 && tailLen >= 20 && slope >= a->minBranchTailSlope) abort_ = 1;
        if (abort_) {
          *aEnd = step * msLen;
          *tEnd = step * (msLen + msD);
          if (step > 0) set_right_delta(a, msE, msD);
          else set_left_delta(a, msE, msD, leftover, tEnd, n);
          *toEnd = 0;
          return msE;
        }
        if (step > 0) {
          /* Force the last error to be a mismatch (forward.C:215-221). */
          if (row == m && 1 + prev[d + 1] == cur[d] && d < right) {
            d++;
            cur[d] = cur[d - 1];
          }
          *aEnd = row;
          *tEnd = row + d;
          set_right_delta(a, e, d);
        } else {
          *aEnd = -row;
          *tEnd = -row - d;
          set_left_delta(a, e, d, leftover, tEnd, n);
        }
        *toEnd = 1;
        return e;
      }
    }

    /* Narrow the band (forward.C:245-280, reverse.C:260-295). */
    while (left <= right && left < 0 && prune(a, e, cur[left], 0)) left++;
    if (left >= 0)
      while (left <= right && prune(a, e, cur[left], left)) left++;
    if (left > right)
      break;
    while (right > 0 && prune(a, e, cur[right], right)) right--;
    if (right <= 0)
      while (prune(a, e, cur[right], 0)) right--;

    for (d = left; d <= right; d++)
      if (cur[d] > longest) {
        bestD   = d;
        bestE   = e;
        longest = cur[d];
      }
    double score = longest * BMV - e;
    if (score > maxScore) {
      maxScore = score;
      msLen    = longest;
      msD      = bestD;
      msE      = bestE;
    }
  }

  *aEnd = step * msLen;
  *tEnd = step * (msLen + msD);
  if (step > 0) set_right_delta(a, msE, msD);
  else set_left_delta(a, msE, msD, leftover, tEnd, n);
  *toEnd = 0;
  return msE;
}

/* Extend_Alignment (prefixEditDistance-extend.C:36-183). */
static int extend_alignment(oic_port_aligner *a, int32_t mStart, int32_t mOffset, int32_t mLen,
                            const char *S, int32_t sLen, const char *T, int32_t tLen, int32_t *sLo,
                            int32_t *sHi, int32_t *tLo, int32_t *tHi, int32_t *errors) {
  int32_t rightErrors = 0, leftErrors = 0, leftover = 0;
  int     rToEnd = 1, lToEnd = 1;
  int32_t sLeftBegin = mStart - 1, sRightBegin = mStart + mLen, sRightLen = sLen - sRightBegin;
  int32_t tLeftBegin = mOffset - 1, tRightBegin = mOffset + mLen, tRightLen = tLen - tRightBegin;
  int32_t totalOlap  = imin(mStart, mOffset) + mLen + imin(sRightLen, tRightLen);
  int32_t errorLimit = a->errorBound[totalOlap];

  a->leftDeltaLen = a->rightDeltaLen = 0;

  if (sRightLen == 0 || tRightLen == 0) {
    *sHi = *tHi = 0;
    rToEnd     = 1;
  } else if (sRightLen <= tRightLen) {
    rightErrors = prefix_dp(a, +1, S + sRightBegin, sRightLen, T + tRightBegin, tRightLen, errorLimit, sHi, tHi,
                            NULL, &rToEnd);
    for (int32_t i = 0; i < a->rightDeltaLen; i++)
      a->rightDelta[i] = -a->rightDelta[i];
  } else {
    rightErrors = prefix_dp(a, +1, T + tRightBegin, tRightLen, S + sRightBegin, sRightLen, errorLimit, tHi, sHi,
                            NULL, &rToEnd);
  }
  *sHi += sRightBegin - 1;
  *tHi += tRightBegin - 1;

  if (sLeftBegin < 0 || tLeftBegin < 0) {
    *sLo = *tLo = 0;
    lToEnd     = 1;
  } else if (sRightBegin <= tRightBegin) {
    leftErrors = prefix_dp(a, -1, S + sLeftBegin, sLeftBegin + 1, T + tLeftBegin, tLeftBegin + 1,
                           errorLimit - rightErrors, sLo, tLo, &leftover, &lToEnd);
  } else {
    leftErrors = prefix_dp(a, -1, T + tLeftBegin, tLeftBegin + 1, S + sLeftBegin, sLeftBegin + 1,
                           errorLimit - rightErrors, tLo, sLo, &leftover, &lToEnd);
    for (int32_t i = 0; i < a->leftDeltaLen; i++)
      a->leftDelta[i] = -a->leftDelta[i];
  }
  *sLo += sLeftBegin + 1;
  *tLo += tLeftBegin + 1;
  *errors = leftErrors + rightErrors;

  int kind = (!rToEnd) ? ((!lToEnd) ? OLAP_NONE : OLAP_RIGHT_BRANCH_PT)
                       : ((!lToEnd) ? OLAP_LEFT_BRANCH_PT : OLAP_DOVETAIL);

  if (a->rightDeltaLen > 0) {
    if (a->rightDelta[0] > 0)
      a->leftDelta[a->leftDeltaLen++] = -(a->rightDelta[0] + leftover + mLen);
    else
      a->leftDelta[a->leftDeltaLen++] = -(a->rightDelta[0] - leftover - mLen);
  }
  for (int32_t i = 1; i < a->rightDeltaLen; i++)
    a->leftDelta[a->leftDeltaLen++] = -a->rightDelta[i];
  a->rightDeltaLen = 0;
  return kind;
}

int oic_port_extend(oic_port_aligner *a, const char *S, int32_t sLen, const char *T, int32_t tLen,
                    int32_t start, int32_t offset, int32_t len, int32_t *out, int32_t *delta,
                    int32_t *deltaLen, uint64_t *cells, uint64_t *slides) {
  uint64_t c0 = a->cells, s0 = a->slides;
  int kind = extend_alignment(a, start, offset, len, S, sLen, T, tLen, &out[0], &out[1], &out[2], &out[3], &out[4]);
  *deltaLen = a->leftDeltaLen;
  if (delta)
    memcpy(delta, a->leftDelta, sizeof(int32_t) * (size_t)a->leftDeltaLen);
  if (cells) *cells += a->cells - c0;
  if (slides) *slides += a->slides - s0;
  return kind;
}

/* ------------------------------------------------------------------------------ */
/* The hash block.  Build_Hash_Index (overlapInCore-Build_Hash_Index.C:414-631),
 * Put_String_In_Hash (:329-404), Hash_Insert (:265-321), Mark_Skip_Kmers (:184-257),
 * Hash_Mark_Empty (:130-177), Mark_Screened_Ends_* (:96-121).                      */

typedef struct kmer_entry {
  uint64_t key;
  uint64_t occBgn;       /* first occurrence in occ[], insertion order */
  uint32_t occCnt;
  uint32_t empty;        /* screened by the -k skip list */
  uint32_t firstStr;     /* block string that inserted it first */
  uint32_t pad;
} kmer_entry;

/* One partition of the k-mer map: keys are spread over partitions so that the block
 * can be built by one thread per partition; each partition still sees its k-mers in
 * the reference's insertion order. */
typedef struct part_map {
  uint64_t    mapCap;         /* power of two */
  int64_t    *map;            /* slot -> entry index or -1 */
  kmer_entry *ent;
  uint64_t    nEnt, entCap;
} part_map;

typedef struct hash_block {
  uint32_t    firstID;        /* Hash_String_Num_Offset */
  uint32_t    nStrings;       /* String_Ct */
  int64_t    *start;          /* String_Start, -1 for an empty entry */
  uint32_t   *length;         /* String_Info.length */
  uint8_t    *lScreened, *rScreened;
  char       *bases;          /* lowercase, NUL after each read */
  uint64_t    basesLen;
  int         nParts;
  part_map   *part;
  uint64_t   *occ;            /* (string << 32) | offset, grouped per entry, insertion order */
  uint64_t    nOcc;
  uint64_t    nDistinct;
} hash_block;

static uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return x;
}

static int part_of(const hash_block *h, uint64_t key) {
  return (int)((mix64(key ^ 0x5bd1e9955bd1e995ULL) >> 20) % (uint64_t)h->nParts);
}

static int64_t pm_find(const part_map *m, uint64_t key) {
  if (m->mapCap == 0) return -1;
  uint64_t msk = m->mapCap - 1, s = mix64(key) & msk;
  while (m->map[s] >= 0) {
    if (m->ent[m->map[s]].key == key)
      return m->map[s];
    s = (s + 1) & msk;
  }
  return -1;
}

static void pm_grow(part_map *m) {
  uint64_t nc = m->mapCap ? m->mapCap * 2 : (1u << 16);
  int64_t *nm = (int64_t *)xmalloc(sizeof(int64_t) * nc);
  memset(nm, 0xff, sizeof(int64_t) * nc);
  for (uint64_t i = 0; i < m->nEnt; i++) {
    uint64_t s = mix64(m->ent[i].key) & (nc - 1);
    while (nm[s] >= 0) s = (s + 1) & (nc - 1);
    nm[s] = (int64_t)i;
  }
  free(m->map);
  m->map    = nm;
  m->mapCap = nc;
}

/* Find-or-create; returns the entry index and sets *created. */
static int64_t pm_insert(part_map *m, uint64_t key, uint32_t str, int *created) {
  if ((m->nEnt + 1) * 2 > m->mapCap)
    pm_grow(m);
  uint64_t msk = m->mapCap - 1, s = mix64(key) & msk;
  while (m->map[s] >= 0) {
    if (m->ent[m->map[s]].key == key) {
      *created = 0;
      return m->map[s];
    }
    s = (s + 1) & msk;
  }
  if (m->nEnt == m->entCap) {
    m->entCap = m->entCap ? m->entCap * 2 : (1u << 16);
    m->ent    = (kmer_entry *)xrealloc(m->ent, sizeof(kmer_entry) * m->entCap);
  }
  kmer_entry *e = &m->ent[m->nEnt];
  memset(e, 0, sizeof(*e));
  e->key      = key;
  e->firstStr = str;
  m->map[s]   = (int64_t)m->nEnt;
  *created    = 1;
  return (int64_t)m->nEnt++;
}

/* The entry of a k-mer in the loaded block, or NULL.  Entries first created by a read
 * past the block's end are not part of the block. */
static kmer_entry *block_find(const hash_block *h, uint64_t key) {
  part_map *m = &h->part[part_of(h, key)];
  int64_t   i = pm_find(m, key);
  if (i < 0) return NULL;
  kmer_entry *e = &m->ent[i];
  return (e->firstStr < h->nStrings) ? e : NULL;
}

static int base_code(char c) {  /* Bit_Equivalent / Char_Is_Bad (overlapInCore.C:500-512) */
  switch (c) {
    case 'a': return 0;
    case 'c': return 1;
    case 'g': return 2;
    case 't': return 3;
    default:  return -1;
  }
}

static void free_block(hash_block *h) {
  free(h->start);
  free(h->length);
  free(h->lScreened);
  free(h->rScreened);
  free(h->bases);
  for (int i = 0; i < h->nParts; i++) {
    free(h->part[i].map);
    free(h->part[i].ent);
  }
  free(h->part);
  free(h->occ);
  memset(h, 0, sizeof(*h));
}

/* Walk the ACGT-only k-mers of string si in order (Put_String_In_Hash :329-404),
 * calling fn for those of partition `part`. */
#define FOR_KMERS_OF_PART(h, si, K, part, BODY)                                       \
  do {                                                                                \
    const char *s_   = (h)->bases + (h)->start[si];                                   \
    uint32_t    len_ = (h)->length[si];                                               \
    uint64_t    key  = 0, msk_ = ((K) >= 32) ? ~0ULL : ((1ULL << (2 * (K))) - 1);     \
    uint32_t    bad_ = 0;                                                             \
    for (uint32_t i_ = 0; i_ < len_; i_++) {                                          \
      int c_ = base_code(s_[i_]);                                                     \
      key    = ((key >> 2) | ((uint64_t)(c_ < 0 ? 0 : c_) << (2 * ((K) - 1)))) & msk_; \
      if (c_ < 0) bad_ = (K);                                                         \
      else if (bad_ > 0) bad_--;                                                      \
      if (i_ + 1 < (K) || bad_ > 0) continue;                                         \
      if (part_of((h), key) != (part)) continue;                                      \
      uint32_t off = i_ + 1 - (K);                                                    \
      BODY                                                                            \
    }                                                                                 \
  } while (0)

/* Hash_Mark_Empty (:130-177) with Mark_Screened_Ends_Chain (:96-121). */
static void mark_empty(hash_block *h, uint64_t key, uint32_t K, int hopeless) {
  kmer_entry *e = block_find(h, key);
  if (e) {
    if (!e->empty) {
      for (uint32_t j = 0; j < e->occCnt; j++) {
        uint64_t o   = h->occ[e->occBgn + j];
        uint32_t sn  = (uint32_t)(o >> 32);
        uint64_t off = (uint32_t)o;
        if (off < HOPELESS_MATCH)
          h->lScreened[sn] = 1;
        if ((uint64_t)h->length[sn] - off - K + 1 < HOPELESS_MATCH)
          h->rScreened[sn] = 1;
      }
    }
    e->empty = 1;
    return;
  }
  if (hopeless) {  /* Add_Extra_Hash_String (:26-86): an empty entry that only screens */
    int       created;
    part_map *m  = &h->part[part_of(h, key)];
    int64_t   ei = pm_insert(m, key, 0, &created);
    m->ent[ei].firstStr = 0;
    m->ent[ei].occCnt   = 0;
    m->ent[ei].empty    = 1;
  }
}

static int read_skip_file(hash_block *h, const char *path, uint32_t K, int hopeless) {
  FILE *F = fopen(path, "r");
  if (!F) {
    fprintf(stderr, "oic_port: cannot open -k file '%s'\n", path);
    return 1;
  }
  char line[1024];
  while (fgets(line, sizeof(line), F)) {
    if (line[0] == '>' && !fgets(line, sizeof(line), F))
      break;
    for (int i = 0; line[i]; i++)
      if (line[i] == ' ' || line[i] == '\t' || line[i] == '\n' || line[i] == '\r') line[i] = 0;
    if (strlen(line) != K) {
      fprintf(stderr, "Short kmer skip kmer '%s', expecting length %u\n", line, K);
      fclose(F);
      return 1;
    }
    uint64_t fw = 0, rc = 0;
    for (uint32_t i = 0; i < K; i++) {
      int c = base_code((char)tolower((unsigned char)line[i]));
      if (c < 0) {
        fprintf(stderr, "oic_port: skip k-mer '%s' is not ACGT\n", line);
        fclose(F);
        return 1;
      }
      fw |= (uint64_t)c << (2 * i);
      rc |= (uint64_t)(3 - c) << (2 * (K - 1 - i));
    }
    mark_empty(h, fw, K, hopeless);
    mark_empty(h, rc, K, hopeless);
  }
  fclose(F);
  return 0;
}

/* Build_Hash_Index (:414-631) with one thread per key partition.  The reference loads
 * reads while the loaded length and the distinct-k-mer count are under their limits
 * (:504-506); here every read under the length limit is scanned, the distinct k-mers
 * each read adds are counted, and the block ends where the reference's loop would
 * stop.  Returns the last read ID loaded, or 0 on error. */
static uint32_t build_block(hash_block *h, const oic_port_params *p, const oic_seqdb *db, uint32_t bgnID,
                            uint32_t endID, uint64_t maxDataLen, int nThreads, int *err) {
  uint32_t K         = p->kmerLen;
  uint64_t tableSize = (uint64_t)1 << p->hashBits;
  uint64_t entryLim  = (uint64_t)(p->maxHashLoad * (double)tableSize * ENTRIES_PER_BUCKET);
  memset(h, 0, sizeof(*h));
  h->firstID = bgnID;
  h->nParts  = nThreads < 1 ? 1 : nThreads;
  h->part    = (part_map *)xcalloc((size_t)h->nParts, sizeof(part_map));

  /* Candidate reads under the length limit (:458-477, :504-545). */
  uint64_t maxAlloc = 0;
  for (uint32_t id = bgnID; maxAlloc < maxDataLen && id <= endID; id++) {
    const oic_seqdb_entry *r = &db->index[id - 1];
    if (r->libID < p->minLibToHash || r->libID > p->maxLibToHash) continue;
    if ((int64_t)r->length < (int64_t)p->minOlapLen) continue;
    maxAlloc += r->length + 1;
  }
  uint64_t nIDs = (uint64_t)endID - bgnID + 1;
  h->start      = (int64_t *)xmalloc(sizeof(int64_t) * nIDs);
  h->length     = (uint32_t *)xcalloc(nIDs, sizeof(uint32_t));
  h->lScreened  = (uint8_t *)xcalloc(nIDs, 1);
  h->rScreened  = (uint8_t *)xcalloc(nIDs, 1);
  h->bases      = (char *)xmalloc(maxAlloc + 1);
  uint64_t total = 0;
  uint32_t nCand = 0;
  for (uint32_t cur = bgnID; total < maxDataLen && cur <= endID; cur++, nCand++) {
    uint32_t               si = nCand;
    const oic_seqdb_entry *r  = &db->index[cur - 1];
    h->start[si]              = -1;
    h->length[si]             = 0;
    h->lScreened[si] = h->rScreened[si] = 1;
    if (r->libID < p->minLibToHash || r->libID > p->maxLibToHash) continue;
    if ((int64_t)r->length < (int64_t)p->minOlapLen) continue;
    if (r->length < K) {
      fprintf(stderr, "oic_port: read %u is shorter than the k-mer size\n", cur);
      *err = 1;
      return 0;
    }
    h->start[si]  = (int64_t)total;
    h->length[si] = r->length;
    h->lScreened[si] = h->rScreened[si] = 0;
    const char *src = db->bases + r->offset;
    for (uint32_t i = 0; i < r->length; i++)
      h->bases[total++] = (char)tolower((unsigned char)src[i]);
    h->bases[total++] = 0;
  }
  h->basesLen = total;

  /* Insert every candidate's k-mers, counting the new keys each read brings. */
  const int P       = h->nParts;
  uint32_t *newKeys = (uint32_t *)xcalloc((size_t)P * nCand + 1, sizeof(uint32_t));
#pragma omp parallel for num_threads(P) schedule(static, 1)
  for (int t = 0; t < P; t++) {
    part_map *m = &h->part[t];
    for (uint32_t si = 0; si < nCand; si++) {
      if (h->start[si] < 0) continue;
      FOR_KMERS_OF_PART(h, si, K, t, {
        int created;
        (void)off;
        pm_insert(m, key, si, &created);
        if (created) newKeys[(size_t)t * nCand + si]++;
      });
    }
  }
  uint64_t len = 0, distinct = 0;
  uint32_t cut;
  for (cut = 0; cut < nCand; cut++) {
    if (!(len < maxDataLen && distinct < entryLim)) break;
    if (h->start[cut] >= 0) len += (uint64_t)h->length[cut] + 1;
    for (int t = 0; t < P; t++) distinct += newKeys[(size_t)t * nCand + cut];
  }
  free(newKeys);
  h->nStrings  = cut;
  h->nDistinct = distinct;
  for (uint32_t si = cut; si < nCand; si++) h->start[si] = -1;

  /* Occurrences of the loaded reads, per entry in insertion order. */
#pragma omp parallel for num_threads(P) schedule(static, 1)
  for (int t = 0; t < P; t++) {
    part_map *m = &h->part[t];
    for (uint64_t i = 0; i < m->nEnt; i++) m->ent[i].occCnt = 0;
    for (uint32_t si = 0; si < cut; si++) {
      if (h->start[si] < 0) continue;
      FOR_KMERS_OF_PART(h, si, K, t, {
        (void)off;
        m->ent[pm_find(m, key)].occCnt++;
      });
    }
  }
  uint64_t acc = 0;
  for (int t = 0; t < P; t++) {
    part_map *m = &h->part[t];
    for (uint64_t i = 0; i < m->nEnt; i++) {
      m->ent[i].occBgn = acc;
      acc += m->ent[i].occCnt;
      m->ent[i].occCnt = 0;
    }
  }
  h->nOcc = acc;
  h->occ  = (uint64_t *)xmalloc(sizeof(uint64_t) * (acc ? acc : 1));
#pragma omp parallel for num_threads(P) schedule(static, 1)
  for (int t = 0; t < P; t++) {
    part_map *m = &h->part[t];
    for (uint32_t si = 0; si < cut; si++) {
      if (h->start[si] < 0) continue;
      FOR_KMERS_OF_PART(h, si, K, t, {
        kmer_entry *e = &m->ent[pm_find(m, key)];
        h->occ[e->occBgn + e->occCnt++] = ((uint64_t)si << 32) | off;
      });
    }
  }

  if (p->kmerSkipFile && read_skip_file(h, p->kmerSkipFile, K, p->useHopelessCheck)) {
    *err = 1;
    return 0;
  }
  *err = 0;
  return bgnID + cut - 1;
}

/* ------------------------------------------------------------------------------ */
/* Per-ref-read work: Find_Overlaps (overlapInCore-Find_Overlaps.C:234-336),
 * Add_Ref (:104-163), Add_Match (:25-96), Process_String_Olaps and Process_Matches
 * (overlapInCore-Process_String_Overlaps.C:354-690), Output_Overlap and
 * Output_Partial_Overlap (overlapInCore-Output.C:26-264).                          */

typedef struct match_node { int32_t offset, len, start, next; } match_node;  /* prefixEditDistance.H:57-62 */

typedef struct pair_rec {
  uint32_t strNum;
  int32_t  matchList;
  int32_t  diagCt, diagBgn, diagEnd;
  int32_t  consistent;
} pair_rec;

typedef struct olap_info {
  int32_t s_lo, s_hi, t_lo, t_hi;
  double  quality;
  int32_t delta_ct;
  int32_t s_left_boundary, s_right_boundary, t_left_boundary, t_right_boundary;
  int32_t min_diag, max_diag;
} olap_info;

typedef struct work_area {
  oic_port_aligner *al;
  match_node       *node;
  int32_t           nodeCap, nodeLen;
  pair_rec         *pair;
  int32_t           pairCap, nPairs;
  int32_t          *pmap;   /* open-addressing T -> pair index */
  int32_t           pmapCap;
  int               leftScreened, rightScreened;
  oic_port_record  *rec;
  uint64_t          nRec, recCap;
  oic_port_stats    st;
  char             *bases;
} work_area;

static int32_t pair_for(work_area *w, uint32_t strNum) {
  if ((w->nPairs + 1) * 2 > w->pmapCap) {
    int32_t nc = w->pmapCap ? w->pmapCap * 2 : 1024;
    free(w->pmap);
    w->pmap    = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)nc);
    w->pmapCap = nc;
    memset(w->pmap, 0xff, sizeof(int32_t) * (size_t)nc);
    for (int32_t i = 0; i < w->nPairs; i++) {
      uint32_t s = (uint32_t)mix64(w->pair[i].strNum) & (uint32_t)(nc - 1);
      while (w->pmap[s] >= 0) s = (s + 1) & (uint32_t)(nc - 1);
      w->pmap[s] = i;
    }
  }
  uint32_t m = (uint32_t)w->pmapCap - 1, s = (uint32_t)mix64(strNum) & m;
  while (w->pmap[s] >= 0) {
    if (w->pair[w->pmap[s]].strNum == strNum)
      return w->pmap[s];
    s = (s + 1) & m;
  }
  if (w->nPairs == w->pairCap) {
    w->pairCap = w->pairCap ? w->pairCap * 2 : 256;
    w->pair    = (pair_rec *)xrealloc(w->pair, sizeof(pair_rec) * (size_t)w->pairCap);
  }
  pair_rec *pr   = &w->pair[w->nPairs];
  pr->strNum     = strNum;
  pr->matchList  = 0;
  pr->diagCt     = 0;
  pr->diagBgn    = (int32_t)AS_MAX_READLEN;
  pr->diagEnd    = 0;
  pr->consistent = 1;
  w->pmap[s]     = w->nPairs;
  return w->nPairs++;
}

/* Add_Match (Find_Overlaps.C:25-96). */
static void add_match(work_area *w, uint32_t tOff, int32_t *head, int32_t offset, int32_t *consistent, int32_t K) {
  int32_t *p, save;
  int32_t  diag = 0, newDiag = (int32_t)tOff - offset, expected = 0, checked = 0, mtf = 0;
  for (p = head; *p != 0; p = &w->node[*p].next) {
    match_node *n = &w->node[*p];
    expected      = n->start + n->len - K + 1;
    diag          = n->offset - n->start;
    if (expected < offset)
      break;
    if (expected == offset) {
      if (newDiag == diag) {
        n->len += 1;
        if (mtf) {
          save              = *p;
          *p                = n->next;
          w->node[save].next = *head;
          *head             = save;
        }
        return;
      } else
        mtf = 1;
    }
    checked++;
  }
  if (w->nodeLen == w->nodeCap) {
    w->nodeCap *= 2;
    w->node = (match_node *)xrealloc(w->node, sizeof(match_node) * (size_t)w->nodeCap);
  }
  if (*head != 0 && (checked > 0 || abs(diag - newDiag) > 3 || offset < expected + K - 2))
    *consistent = 0;
  save           = *head;
  *head          = w->nodeLen++;
  match_node *nn = &w->node[*head];
  nn->offset     = (int32_t)tOff;
  nn->len        = K;
  nn->start      = offset;
  nn->next       = save;
}

/* Add_Overlap (Process_String_Overlaps.C:175-244). */
static void add_overlap(int partial, int32_t s_lo, int32_t s_hi, int32_t t_lo, int32_t t_hi, double q,
                        int32_t deltaCt, olap_info *o, int *ct) {
  if (!partial) {
    int32_t nd = t_lo - s_lo;
    for (int i = 0; i < *ct; i++) {
      int32_t od = o[i].t_lo - o[i].s_lo;
      if ((nd > 0 && od > 0 && o[i].t_right_boundary - nd - o[i].s_left_boundary >= MIN_INTERSECTION) ||
          (nd <= 0 && od <= 0 && o[i].s_right_boundary + nd - o[i].t_left_boundary >= MIN_INTERSECTION)) {
        if (nd < o[i].min_diag) o[i].min_diag = nd;
        if (nd > o[i].max_diag) o[i].max_diag = nd;
        if (s_lo < o[i].s_left_boundary) o[i].s_left_boundary = s_lo;
        if (s_hi > o[i].s_right_boundary) o[i].s_right_boundary = s_hi;
        if (t_lo < o[i].t_left_boundary) o[i].t_left_boundary = t_lo;
        if (t_hi > o[i].t_right_boundary) o[i].t_right_boundary = t_hi;
        if (q < o[i].quality) {
          o[i].s_lo     = s_lo;
          o[i].s_hi     = s_hi;
          o[i].t_lo     = t_lo;
          o[i].t_hi     = t_hi;
          o[i].quality  = q;
          o[i].delta_ct = deltaCt;
        }
        return;
      }
    }
  }
  if (*ct >= MAX_DISTINCT_OLAPS)
    return;
  olap_info *n = &o[*ct];
  n->s_lo = n->s_left_boundary = s_lo;
  n->s_hi = n->s_right_boundary = s_hi;
  n->t_lo = n->t_left_boundary = t_lo;
  n->t_hi = n->t_right_boundary = t_hi;
  n->quality  = q;
  n->delta_ct = deltaCt;
  n->min_diag = n->max_diag = t_lo - s_lo;
  (*ct)++;
}

/* Lies_On_Alignment (Process_String_Overlaps.C:260-281). */
static int lies_on_alignment(const int32_t *delta, int32_t deltaLen, int32_t start, int32_t offset, int32_t s_lo,
                             int32_t t_lo) {
  int32_t diag = t_lo - s_lo, nd = offset - start;
  for (int32_t i = 0; i < deltaLen; i++) {
    s_lo += abs(delta[i]);
    if (start < s_lo)
      return abs(nd - diag) <= SHIFT_SLACK;
    if (delta[i] < 0)
      diag++;
    else {
      s_lo++;
      diag--;
    }
  }
  return abs(nd - diag) <= SHIFT_SLACK;
}

/* Combine_Into_One_Olap (:40-96). */
static void combine_into_one(olap_info *o, int ct, int *deleted) {
  int best = 0;
  int32_t mnd = o[0].min_diag, mxd = o[0].max_diag, slb = o[0].s_left_boundary, srb = o[0].s_right_boundary,
          tlb = o[0].t_left_boundary, trb = o[0].t_right_boundary;
  for (int i = 1; i < ct; i++) {
    int32_t li = 1 + imin(o[i].s_hi - o[i].s_lo, o[i].t_hi - o[i].t_lo);
    int32_t lb = 1 + imin(o[best].s_hi - o[best].s_lo, o[best].t_hi - o[best].t_lo);
    if (o[i].quality < o[best].quality || (o[i].quality == o[best].quality && li > lb))
      best = i;
    if (o[i].min_diag < mnd) mnd = o[i].min_diag;
    if (o[i].max_diag > mxd) mxd = o[i].max_diag;
    if (o[i].s_left_boundary < slb) slb = o[i].s_left_boundary;
    if (o[i].s_right_boundary > srb) srb = o[i].s_right_boundary;
    if (o[i].t_left_boundary < tlb) tlb = o[i].t_left_boundary;
    if (o[i].t_right_boundary > trb) trb = o[i].t_right_boundary;
  }
  o[best].min_diag = mnd;
  o[best].max_diag = mxd;
  o[best].s_left_boundary  = slb;
  o[best].s_right_boundary = srb;
  o[best].t_left_boundary  = tlb;
  o[best].t_right_boundary = trb;
  for (int i = 0; i < ct; i++)
    deleted[i] = (i != best);
}

/* Merge_Intersecting_Olaps (:106-162). */
static void merge_intersecting(olap_info *p, int ct, int *deleted) {
  for (int i = 0; i < ct - 1; i++)
    for (int j = i + 1; j < ct; j++) {
      if (deleted[i] || deleted[j]) continue;
      int32_t lo = p[i].min_diag, hi = p[i].max_diag;
      if ((lo <= 0 && p[j].min_diag > 0) || (lo > 0 && p[j].min_diag <= 0)) continue;
      if ((lo >= 0 && p[j].t_right_boundary - lo - p[j].s_left_boundary >= MIN_INTERSECTION) ||
          (lo <= 0 && p[j].s_right_boundary + lo - p[j].t_left_boundary >= MIN_INTERSECTION) ||
          (hi >= 0 && p[j].t_right_boundary - hi - p[j].s_left_boundary >= MIN_INTERSECTION) ||
          (hi <= 0 && p[j].s_right_boundary + hi - p[j].t_left_boundary >= MIN_INTERSECTION)) {
        olap_info *keep, *disc;
        if (p[i].quality < p[j].quality) { keep = p + i; disc = p + j; deleted[j] = 1; }
        else { keep = p + j; disc = p + i; deleted[i] = 1; }
        if (disc->min_diag < keep->min_diag) keep->min_diag = disc->min_diag;
        if (disc->max_diag > keep->max_diag) keep->max_diag = disc->max_diag;
        if (disc->s_left_boundary < keep->s_left_boundary) keep->s_left_boundary = disc->s_left_boundary;
        if (disc->s_right_boundary > keep->s_right_boundary) keep->s_right_boundary = disc->s_right_boundary;
        if (disc->t_left_boundary < keep->t_left_boundary) keep->t_left_boundary = disc->t_left_boundary;
        if (disc->t_right_boundary > keep->t_right_boundary) keep->t_right_boundary = disc->t_right_boundary;
      }
    }
}

/* Choose_Best_Partial (:289-311). */
static void choose_best_partial(olap_info *o, int ct, int *deleted) {
  int    best = 0;
  double mb0  = (1.0 - o[0].quality) * (2 + o[0].s_hi - o[0].s_lo + o[0].t_hi - o[0].t_lo);
  for (int i = 1; i < ct; i++) {
    double mb = (1.0 - o[i].quality) * (2 + o[i].s_hi - o[i].s_lo + o[i].t_hi - o[i].t_lo);
    if (mb0 < mb || (mb0 == mb && o[i].quality < o[best].quality))
      best = i;
  }
  for (int i = 0; i < ct; i++)
    deleted[i] = (i != best);
}

/* ovOverlap encoding (src/stores/ovOverlap.H:31-78,162-166,204; AS_MAX_READLEN_BITS 21). */
static uint32_t encode_evalue(double q) {
  return (q < 65535 / 100000.0) ? (uint32_t)(100000.0 * q + 0.5) : 65535u;
}

static void emit(work_area *w, uint32_t a, uint32_t b, uint32_t ahg5, uint32_t ahg3, uint32_t bhg5, uint32_t bhg3,
                 uint32_t span, uint32_t evalue, uint32_t flipped, uint32_t forOBT, uint32_t forDUP, uint32_t forUTG) {
  const uint64_t M21 = (1u << 21) - 1;
  uint64_t d0 = ((uint64_t)ahg5 & M21) | (((uint64_t)ahg3 & M21) << 21) | (((uint64_t)evalue & 0xffff) << 42) |
                ((uint64_t)(flipped & 1) << 58) | ((uint64_t)(forOBT & 1) << 59) | ((uint64_t)(forDUP & 1) << 60) |
                ((uint64_t)(forUTG & 1) << 61);
  uint64_t d1 = ((uint64_t)bhg5 & M21) | (((uint64_t)bhg3 & M21) << 21) | (((uint64_t)span & M21) << 42);
  if (w->nRec == w->recCap) {
    w->recCap = w->recCap ? w->recCap * 2 : 4096;
    w->rec    = (oic_port_record *)xrealloc(w->rec, sizeof(oic_port_record) * w->recCap);
  }
  oic_port_record *r = &w->rec[w->nRec++];
  r->w[0] = a;
  r->w[1] = b;
  r->w[2] = (uint32_t)(d0 >> 32);
  r->w[3] = (uint32_t)d0;
  r->w[4] = (uint32_t)(d1 >> 32);
  r->w[5] = (uint32_t)d1;
}

/* The span is accumulated in a 21-bit field, one term at a time (Output.C:41-45). */
static uint32_t span21(const olap_info *o) {
  const uint32_t M21 = (1u << 21) - 1;
  uint32_t sp = (uint32_t)(o->s_hi - o->s_lo) & M21;
  sp          = (sp + (uint32_t)(o->t_hi - o->t_lo)) & M21;
  sp          = (sp + (uint32_t)o->delta_ct) & M21;
  return sp / 2;
}

/* Output_Overlap (Output.C:26-191). */
static void output_overlap(work_area *w, uint32_t sID, int32_t sLen, int dirReverse, uint32_t tID, int32_t tLen,
                           const olap_info *o) {
  uint32_t span = span21(o);
  int32_t  sRH = sLen - o->s_hi - 1, tRH = tLen - o->t_hi - 1;
  int      sLeft = (o->s_lo > o->t_lo) || (o->s_lo == o->t_lo && sRH > tRH);
  uint32_t a = sLeft ? sID : tID, b = sLeft ? tID : sID;
  char     orient;
  int32_t  ahg, bhg;
  if (sLeft) {
    orient = dirReverse ? 'O' : 'N';
    ahg    = o->s_lo;
    bhg    = tRH - sRH;
  } else {
    orient = dirReverse ? 'I' : 'N';
    ahg    = o->t_lo;
    bhg    = sRH - tRH;
  }
  if (orient == 'O' && sRH >= tRH) {
    orient = 'I';
    ahg    = -(tRH - sRH);
    bhg    = -(o->s_lo);
  }
  int32_t ah, bh;
  uint32_t flipped;
  if (orient == 'O') { ah = -bhg; bh = -ahg; flipped = 1; }
  else { ah = ahg; bh = bhg; flipped = (orient == 'I'); }
  uint32_t ahg5 = ah < 0 ? 0 : (uint32_t)ah, bhg5 = ah < 0 ? (uint32_t)-ah : 0;
  uint32_t bhg3 = bh < 0 ? 0 : (uint32_t)bh, ahg3 = bh < 0 ? (uint32_t)-bh : 0;
  emit(w, a, b, ahg5, ahg3, bhg5, bhg3, span, encode_evalue(o->quality), flipped, 0, 0, 1);
  w->st.totalOverlaps++;
  if (bhg <= 0) w->st.containedOverlaps++;
  else w->st.dovetailOverlaps++;
}

/* Output_Partial_Overlap (Output.C:195-264). */
static void output_partial(work_area *w, uint32_t sID, uint32_t tID, int dirReverse, const olap_info *o, int32_t sLen,
                           int32_t tLen) {
  uint32_t span = span21(o);
  uint32_t ahg5, ahg3, bhg5, bhg3;
  if (!dirReverse) {
    ahg5 = (uint32_t)o->s_lo;
    ahg3 = (uint32_t)(sLen - (o->s_hi + 1));
    bhg5 = (uint32_t)o->t_lo;
    bhg3 = (uint32_t)(tLen - (o->t_hi + 1));
  } else {
    ahg5 = (uint32_t)(sLen - (o->s_hi + 1));
    ahg3 = (uint32_t)o->s_lo;
    bhg5 = (uint32_t)(tLen - (o->t_hi + 1));
    bhg3 = (uint32_t)o->t_lo;
  }
  emit(w, sID, tID, ahg5, ahg3, bhg5, bhg3, span, encode_evalue(o->quality), dirReverse ? 1u : 0u, 1, 1, 0);
  w->st.totalOverlaps++;
}

/* Process_Matches (Process_String_Overlaps.C:354-547). */
static void process_matches(work_area *w, const oic_port_params *p, int32_t *start, const char *S, int32_t sLen,
                            uint32_t sID, int dirReverse, const char *T, int32_t tLen, int tLScr, int tRScr,
                            uint32_t tID, int consistent) {
  oic_port_aligner *al = w->al;
  const int32_t     K  = (int32_t)p->kmerLen;
  olap_info         olap[MAX_DISTINCT_OLAPS];
  int               nOlap = 0, nOut = 0;

  if (p->useHopelessCheck && w->node[*start].next == 0 && !p->partial) {
    match_node *m = &w->node[*start];
    int         hopeless = 0;
    int32_t     sHead = m->start, tHead = m->offset;
    if (sHead <= tHead) {
      if (sHead > HOPELESS_MATCH && !w->leftScreened) hopeless = 1;
    } else {
      if (tHead > HOPELESS_MATCH && !tLScr) hopeless = 1;
    }
    int32_t sTail = sLen - sHead - m->len + 1, tTail = tLen - tHead - m->len + 1;
    if (sTail <= tTail) {
      if (sTail > HOPELESS_MATCH && !w->rightScreened) hopeless = 1;
    } else {
      if (tTail > HOPELESS_MATCH && !tRScr) hopeless = 1;
    }
    if (hopeless) {
      *start = 0;
      w->st.kmerHitsWithoutOlap++;
      return;
    }
  }
  (void)K;

  while (*start != 0) {
    int32_t longest = *start, maxLen = w->node[*start].len;
    for (int32_t q = w->node[*start].next; q != 0; q = w->node[q].next)
      if (w->node[q].len > maxLen) {
        maxLen  = w->node[q].len;
        longest = q;
      }
    match_node lm = w->node[longest];
    int32_t    sLo = 0, sHi = 0, tLo = 0, tHi = 0, errors = 0;
    int        kind = extend_alignment(al, lm.start, lm.offset, lm.len, S, sLen, T, tLen, &sLo, &sHi, &tLo, &tHi,
                                       &errors);
    w->st.extensions++;
    if (kind == OLAP_DOVETAIL || p->partial) {
      if (1 + sHi - sLo >= p->minOlapLen && 1 + tHi - tLo >= p->minOlapLen) {
        int32_t olapLen = 1 + imin(sHi - sLo, tHi - tLo);
        double  quality = (double)errors / olapLen;
        if (errors <= al->errorBound[olapLen])
          add_overlap(p->partial, sLo, sHi, tLo, tHi, quality, al->leftDeltaLen, olap, &nOlap);
      }
    }
    if (consistent)
      *start = 0;
    for (int32_t *ref = start; *ref != 0;) {
      match_node *q = &w->node[*ref];
      if (*ref == longest ||
          ((kind == OLAP_DOVETAIL || p->partial) && sLo - SHIFT_SLACK <= q->start &&
           q->start + q->len <= (sHi + 1) + SHIFT_SLACK - 1 &&
           lies_on_alignment(al->leftDelta, al->leftDeltaLen, q->start, q->offset, sLo, tLo)))
        *ref = q->next;
      else
        ref = &q->next;
    }
  }

  if (nOlap > 0) {
    int deleted[MAX_DISTINCT_OLAPS] = {0, 0, 0};
    if (p->partial) {
      if (p->uniqueOlapPerPair) choose_best_partial(olap, nOlap, deleted);
    } else {
      if (p->uniqueOlapPerPair) combine_into_one(olap, nOlap, deleted);
      else merge_intersecting(olap, nOlap, deleted);
    }
    for (int i = 0; i < nOlap; i++)
      if (!deleted[i]) {
        if (p->partial) output_partial(w, sID, tID, dirReverse, &olap[i], sLen, tLen);
        else output_overlap(w, sID, sLen, dirReverse, tID, tLen, &olap[i]);
        nOut++;
      }
  }
  if (nOut == 0)
    w->st.kmerHitsWithoutOlap++;
  else {
    w->st.kmerHitsWithOlap++;
    if (nOut > 1) w->st.multiOverlap++;
  }
}

static void find_overlaps(work_area *w, const oic_port_params *p, const hash_block *h, const char *S, int32_t sLen,
                          uint32_t sID, int dirReverse, double kmerExpectConst) {
  const uint32_t K = p->kmerLen;
  w->nPairs        = 0;
  w->nodeLen       = 1;
  if (w->pmapCap) memset(w->pmap, 0xff, sizeof(int32_t) * (size_t)w->pmapCap);
  w->leftScreened = w->rightScreened = 0;

  uint64_t key = 0, mask = (K >= 32) ? ~0ULL : ((1ULL << (2 * K)) - 1);
  uint32_t bad = 0;
  for (int32_t i = 0; i < sLen; i++) {
    int c = base_code(S[i]);
    key   = ((key >> 2) | ((uint64_t)(c < 0 ? 0 : c) << (2 * (K - 1)))) & mask;
    if (c < 0) bad = K;
    else if (bad > 0) bad--;
    if (i + 1 < (int32_t)K || bad > 0)
      continue;
    int32_t off = i + 1 - (int32_t)K;
    const kmer_entry *e = block_find(h, key);
    if (!e)
      continue;
    if (e->empty) {  /* hi_hits: Find_Overlaps.C:274-276 (offset 0), :310-317 */
      if (off == 0) w->leftScreened = 1;
      else {
        if (off < HOPELESS_MATCH) w->leftScreened = 1;
        if (sLen - off - (int32_t)K + 1 < HOPELESS_MATCH) w->rightScreened = 1;
      }
      continue;
    }
    /* Chain order: newest insertion first (Build_Hash_Index.C:291-294). */
    for (int64_t j = (int64_t)e->occCnt - 1; j >= 0; j--) {
      uint64_t o  = h->occ[e->occBgn + (uint64_t)j];
      uint32_t sn = (uint32_t)(o >> 32);
      if (!((uint64_t)sID < (uint64_t)sn + h->firstID))
        continue;
      w->st.seeds++;
      int32_t   pi = pair_for(w, sn);
      pair_rec *pr = &w->pair[pi];
      pr->diagCt++;
      if (pr->diagBgn > off) pr->diagBgn = off;
      if (pr->diagEnd < off) pr->diagEnd = off;
      int32_t cons = pr->consistent;
      add_match(w, (uint32_t)o, &pr->matchList, off, &cons, (int32_t)K);
      w->pair[pi].consistent = cons;
    }
  }

  w->st.candidatePairs += (uint64_t)w->nPairs;
  for (int32_t pi = 0; pi < w->nPairs; pi++) {
    pair_rec *pr = &w->pair[pi];
    if (p->minKmers) {  /* computeMinimumKmers (Process_String_Overlaps.C:21-33) */
      double   ol  = (double)(pr->diagEnd - pr->diagBgn);
      if (ol < 0) ol = -ol;
      uint64_t exp_ = (ol < (double)K) ? 0 : (uint64_t)(int)floor(kmerExpectConst * (ol - (double)K + 1));
      uint64_t minK = (uint64_t)p->minKmers;
      uint64_t need = minK > exp_ ? minK : exp_;
      if (need > (uint64_t)pr->diagCt) {
        w->st.kmerHitsSkipped++;
        continue;
      }
    }
    uint32_t sn = pr->strNum;
    process_matches(w, p, &pr->matchList, S, sLen, sID, dirReverse, h->bases + h->start[sn], (int32_t)h->length[sn],
                    h->lScreened[sn], h->rScreened[sn], sn + h->firstID, pr->consistent);
  }
}

static void reverse_complement(char *s, int32_t n) {
  for (int32_t i = 0, j = n - 1; i <= j; i++, j--) {
    char a = s[i], b = s[j];
#define COMP(c) ((c) == 'a' ? 't' : (c) == 'c' ? 'g' : (c) == 'g' ? 'c' : (c) == 't' ? 'a' : (c))
    s[i] = COMP(b);
    s[j] = COMP(a);
#undef COMP
  }
}

static void add_stats(oic_port_stats *d, const oic_port_stats *s) {
  d->kmerHitsWithoutOlap += s->kmerHitsWithoutOlap;
  d->kmerHitsWithOlap += s->kmerHitsWithOlap;
  d->kmerHitsSkipped += s->kmerHitsSkipped;
  d->multiOverlap += s->multiOverlap;
  d->totalOverlaps += s->totalOverlaps;
  d->containedOverlaps += s->containedOverlaps;
  d->dovetailOverlaps += s->dovetailOverlaps;
  d->dpCells += s->dpCells;
  d->slideBases += s->slideBases;
  d->extensions += s->extensions;
  d->seeds += s->seeds;
  d->candidatePairs += s->candidatePairs;
}

static void work_areas_new(work_area **out, int nt, const oic_port_params *p) {
  work_area *wa = (work_area *)xcalloc((size_t)nt, sizeof(work_area));
  for (int t = 0; t < nt; t++) {
    wa[t].al      = oic_port_aligner_new(p->maxErate, p->alignNoise, p->partial);
    wa[t].nodeCap = 10000;
    wa[t].node    = (match_node *)xmalloc(sizeof(match_node) * (size_t)wa[t].nodeCap);
    wa[t].bases   = (char *)xmalloc(AS_MAX_READLEN + 2);
  }
  *out = wa;
}

/* Collect the records and counters of the work areas (and reset them). */
static void work_areas_collect(work_area *wa, int nt, oic_port_record **recs, uint64_t *nRecs, oic_port_stats *stats) {
  for (int t = 0; t < nt; t++) {
    wa[t].st.dpCells    = wa[t].al->cells;
    wa[t].st.slideBases = wa[t].al->slides;
    wa[t].al->cells = wa[t].al->slides = 0;
    add_stats(stats, &wa[t].st);
    memset(&wa[t].st, 0, sizeof(wa[t].st));
    if (wa[t].nRec) {
      *recs = (oic_port_record *)xrealloc(*recs, sizeof(oic_port_record) * (size_t)(*nRecs + wa[t].nRec));
      memcpy(*recs + *nRecs, wa[t].rec, sizeof(oic_port_record) * (size_t)wa[t].nRec);
      *nRecs += wa[t].nRec;
      wa[t].nRec = 0;
    }
  }
}


static void work_areas_free(work_area *wa, int nt) {
  for (int t = 0; t < nt; t++) {
    oic_port_aligner_free(wa[t].al);
    free(wa[t].node);
    free(wa[t].pair);
    free(wa[t].pmap);
    free(wa[t].rec);
    free(wa[t].bases);
  }
  free(wa);
}

/* Process_Overlaps (overlapInCore-Process_Overlaps.C:24-122) for ref IDs [lo, hi]:
 * each ref read forward, then reverse-complemented. */
static void run_refs(const oic_port_params *p, const oic_seqdb *db, const hash_block *h, work_area *wa, int nt,
                     int64_t refLo, int64_t refHi, double kmerExpect) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (int64_t fi = refLo; fi <= refHi; fi++) {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    work_area             *w = &wa[t];
    const oic_seqdb_entry *r = &db->index[fi - 1];
    if (r->libID < p->minLibToRef || r->libID > p->maxLibToRef) continue;
    if ((int64_t)r->length < (int64_t)p->minOlapLen) continue;
    if (r->length < p->kmerLen) continue;
    const char *src = db->bases + r->offset;
    for (uint32_t i = 0; i < r->length; i++)
      w->bases[i] = (char)tolower((unsigned char)src[i]);
    w->bases[r->length] = 0;
    find_overlaps(w, p, h, w->bases, (int32_t)r->length, (uint32_t)fi, 0, kmerExpect);
    reverse_complement(w->bases, (int32_t)r->length);
    find_overlaps(w, p, h, w->bases, (int32_t)r->length, (uint32_t)fi, 1, kmerExpect);
  }
}

static double wall_seconds(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* Checks and derived values shared by the whole-stage run and a session. */
static int prepare_params(oic_port_params *P, const oic_seqdb *db, double *kmerExpect) {
  if (P->kmerLen == 0 || P->kmerLen > 31) {
    fprintf(stderr, "oic_port: k-mer size must be 1..31\n");
    return 1;
  }
  uint32_t last = db->nReads;
  if (P->bgnHashID < 1) P->bgnHashID = 1;
  if (last < P->endHashID) P->endHashID = last;
  if (P->bgnRefID < 1) P->bgnRefID = 1;
  if (P->endRefID > last) P->endRefID = last;
  for (uint32_t i = 0; i < db->nReads; i++)
    if (db->index[i].length > AS_MAX_READLEN) {
      fprintf(stderr, "oic_port: read %u longer than %u\n", i + 1, AS_MAX_READLEN);
      return 1;
    }
  /* A read that passes the length filter but is shorter than k trips an assertion in
   * Find_Overlaps.C:249 (as a ref read) and reads past its own end in
   * Build_Hash_Index.C:347-350 (as a hash read); both are rejected here. */
  for (uint32_t id = 1; id <= last; id++) {
    const oic_seqdb_entry *r = &db->index[id - 1];
    if ((int64_t)r->length >= (int64_t)P->minOlapLen && r->length < P->kmerLen) {
      fprintf(stderr, "oic_port: read %u (length %u) is shorter than the k-mer size %u\n", id, r->length, P->kmerLen);
      return 1;
    }
  }
  *kmerExpect = exp(-1.0 * (double)P->kmerLen * P->maxErate);
  if (P->minKmers)   /* overlapInCore.C:410-411 */
    P->minKmers = (int)floor(*kmerExpect * (double)((uint64_t)(int64_t)P->minOlapLen - P->kmerLen + 1));
  if (P->numThreads < 1) P->numThreads = 1;
  return 0;
}

/* OverlapDriver (overlapInCore.C:161-277). */
int oic_port_run(const oic_port_params *pin, const oic_seqdb *db, oic_port_record **recs, uint64_t *nRecs,
                 oic_port_stats *stats) {
  oic_port_params P = *pin;
  double          kmerExpect;
  memset(stats, 0, sizeof(*stats));
  *recs  = NULL;
  *nRecs = 0;
  if (prepare_params(&P, db, &kmerExpect)) return 1;
  const oic_port_params *p = &P;
  int        nt = (int)P.numThreads;
  work_area *wa;
  work_areas_new(&wa, nt, p);

  /* The ref reads one thread chunk loop visits (Process_Overlaps.C:33; overlapInCore.C:225):
   * every ID in [bgnRef,endRef] except endRef when a chunk would start exactly on it. */
  uint32_t refEnd = P.endRefID;
  if (P.bgnRefID <= P.endRefID) {
    uint32_t perThread = 1 + (P.endRefID - P.bgnRefID) / (uint32_t)nt / 8;
    if ((P.endRefID - P.bgnRefID) % perThread == 0)
      refEnd = P.endRefID - 1;
  }

  int      rc   = 0;
  uint32_t bgnH = P.bgnHashID;
  while (bgnH < P.endHashID && rc == 0) {   /* overlapInCore.C:204 */
    hash_block h;
    int        err  = 0;
    uint32_t   endH = build_block(&h, p, db, bgnH, P.endHashID, P.maxHashDataLen + AS_MAX_READLEN, nt, &err);
    if (err) {
      free_block(&h);
      rc = 1;
      break;
    }
    stats->nHashBlocks++;
    fprintf(stderr, "oic_port: hash block %u-%u (%lu distinct k-mers, %lu occurrences)\n", bgnH, endH,
            (unsigned long)h.nDistinct, (unsigned long)h.nOcc);
    int64_t refLo = P.bgnRefID, refHi = (P.bgnRefID <= P.endRefID) ? (int64_t)refEnd : (int64_t)P.bgnRefID - 1;
    run_refs(p, db, &h, wa, nt, refLo, refHi, kmerExpect);
    free_block(&h);
    bgnH = endH + 1;
  }
  uint32_t nb = stats->nHashBlocks;
  work_areas_collect(wa, nt, recs, nRecs, stats);
  stats->nHashBlocks = nb;
  work_areas_free(wa, nt);
  return rc;
}

struct oic_port_session {
  oic_port_params  P;
  const oic_seqdb *db;
  hash_block       h;
  work_area       *wa;
  int              nt;
  double           kmerExpect;
  uint32_t         lastLoaded;
};

oic_port_session *oic_port_session_new(const oic_port_params *pin, const oic_seqdb *db, double *buildSeconds) {
  oic_port_session *s = (oic_port_session *)xcalloc(1, sizeof(*s));
  s->P  = *pin;
  s->db = db;
  if (prepare_params(&s->P, db, &s->kmerExpect)) {
    free(s);
    return NULL;
  }
  s->nt     = (int)s->P.numThreads;
  double t0 = wall_seconds();
  int    err = 0;
  s->lastLoaded = build_block(&s->h, &s->P, db, s->P.bgnHashID, s->P.endHashID, s->P.maxHashDataLen + AS_MAX_READLEN,
                              s->nt, &err);
  if (buildSeconds) *buildSeconds = wall_seconds() - t0;
  if (err) {
    free_block(&s->h);
    free(s);
    return NULL;
  }
  work_areas_new(&s->wa, s->nt, &s->P);
  return s;
}

uint32_t oic_port_session_last_loaded(const oic_port_session *s) { return s->lastLoaded; }

int oic_port_session_refs(oic_port_session *s, uint32_t bgnRef, uint32_t endRef, oic_port_record **recs,
                          uint64_t *nRecs, oic_port_stats *stats) {
  memset(stats, 0, sizeof(*stats));
  *recs  = NULL;
  *nRecs = 0;
  if (bgnRef < 1) bgnRef = 1;
  if (endRef > s->db->nReads) endRef = s->db->nReads;
  run_refs(&s->P, s->db, &s->h, s->wa, s->nt, bgnRef, endRef, s->kmerExpect);
  work_areas_collect(s->wa, s->nt, recs, nRecs, stats);
  return 0;
}

void oic_port_session_free(oic_port_session *s) {
  if (!s) return;
  work_areas_free(s->wa, s->nt);
  free_block(&s->h);
  free(s);
}

oic_seqdb *oic_port_seqdb_load(const char *path) {
  oic_seqdb *db = (oic_seqdb *)xcalloc(1, sizeof(oic_seqdb));
  if (oic_seqdb_load(path, db)) {
    free(db);
    return NULL;
  }
  return db;
}

void oic_port_seqdb_free(oic_seqdb *db) {
  if (!db) return;
  oic_seqdb_free(db);
  free(db);
}

void oic_port_records_free(oic_port_record *r) { free(r); }
