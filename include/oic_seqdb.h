/*
 * oic_seqdb.h -- the read container read by overlapInCore (GPU build) and by
 * the CPU oracle.
 *
 * canu's own sqStore keeps reads in 2/3-bit encoded blobs whose codec lives in
 * the meryl-utility library; this container carries the same information the
 * overlap stage reads from an sqStore (overlapInCore-Build_Hash_Index.C:460-545,
 * overlapInCore-Process_Overlaps.C:314-334): for each 1-based read ID its
 * library ID, its length and its bases.
 *
 * Layout (little endian):
 *   char     magic[8]      "OICSEQ01"
 *   uint32   nReads
 *   uint32   reserved      0
 *   uint64   nBases        total bases over all reads
 *   struct { uint32 libID; uint32 length; uint64 offset; } index[nReads]
 *   char     bases[nBases] ASCII, read i occupies bases[offset_i .. offset_i+length_i)
 *
 * Read ID r (1-based) is index[r-1].  Bases are A/C/G/T/N in either case.
 *
 * Header-only, C99 and C++ compatible.
 */
#ifndef OIC_SEQDB_H
#define OIC_SEQDB_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oic_seqdb_entry {
  uint32_t libID;
  uint32_t length;
  uint64_t offset;
} oic_seqdb_entry;

typedef struct oic_seqdb {
  uint32_t          nReads;
  uint64_t          nBases;
  oic_seqdb_entry  *index;   /* nReads entries, read r at index[r-1] */
  char             *bases;   /* nBases bytes */
} oic_seqdb;

/* Load a container; returns 0 on success, nonzero (and an empty db) on error. */
static inline int oic_seqdb_load(const char *path, oic_seqdb *db) {
  memset(db, 0, sizeof(*db));
  FILE *F = fopen(path, "rb");
  if (F == NULL)
    return 1;
  char     magic[8];
  uint32_t hdr[2];
  uint64_t nb;
  if (fread(magic, 1, 8, F) != 8 || memcmp(magic, "OICSEQ01", 8) != 0 ||
      fread(hdr, 4, 2, F) != 2 || fread(&nb, 8, 1, F) != 1) {
    fclose(F);
    return 2;
  }
  db->nReads = hdr[0];
  db->nBases = nb;
  db->index  = (oic_seqdb_entry *)malloc(sizeof(oic_seqdb_entry) * (size_t)(db->nReads + 1));
  db->bases  = (char *)malloc((size_t)nb + 1);
  if (db->index == NULL || db->bases == NULL ||
      fread(db->index, sizeof(oic_seqdb_entry), db->nReads, F) != db->nReads ||
      fread(db->bases, 1, (size_t)nb, F) != (size_t)nb) {
    fclose(F);
    free(db->index);
    free(db->bases);
    memset(db, 0, sizeof(*db));
    return 3;
  }
  db->bases[nb] = 0;
  fclose(F);
  for (uint32_t i = 0; i < db->nReads; i++)
    if (db->index[i].offset + db->index[i].length > nb) {
      free(db->index);
      free(db->bases);
      memset(db, 0, sizeof(*db));
      return 4;
    }
  return 0;
}

static inline void oic_seqdb_free(oic_seqdb *db) {
  free(db->index);
  free(db->bases);
  memset(db, 0, sizeof(*db));
}

/* Write a container from parallel arrays (reads concatenated in `bases`). */
static inline int oic_seqdb_write(const char *path, uint32_t nReads, const uint32_t *libID,
                                  const uint32_t *lengths, const char *bases) {
  FILE *F = fopen(path, "wb");
  if (F == NULL)
    return 1;
  uint64_t nb = 0;
  for (uint32_t i = 0; i < nReads; i++)
    nb += lengths[i];
  uint32_t hdr[2] = {nReads, 0};
  int      bad    = (fwrite("OICSEQ01", 1, 8, F) != 8) || (fwrite(hdr, 4, 2, F) != 2) ||
             (fwrite(&nb, 8, 1, F) != 1);
  uint64_t off = 0;
  for (uint32_t i = 0; i < nReads && !bad; i++) {
    oic_seqdb_entry e = {libID ? libID[i] : 1u, lengths[i], off};
    bad |= (fwrite(&e, sizeof(e), 1, F) != 1);
    off += lengths[i];
  }
  if (!bad && nb > 0)
    bad |= (fwrite(bases, 1, (size_t)nb, F) != (size_t)nb);
  bad |= (fclose(F) != 0);
  return bad ? 2 : 0;
}

#ifdef __cplusplus
}
#endif

#endif
