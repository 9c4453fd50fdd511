/*
 * oic_ovfile.h -- the overlapper's output files, as canu's ovFile writes and reads them
 * (part of liboic_gpu.so; host code only, no GPU needed).
 *
 * <name>.ovb   ovFile(ovFileFullWrite) (src/stores/ovStoreFile.C:98-121, 212-286): the
 *              records are buffered in blocks of at most 262,080 uint32 words (a whole
 *              number of records) and each block is written as [uint64 compressed
 *              length][raw snappy block].  A record is six uint32 words: a_iid, b_iid,
 *              dat[0] >> 32, dat[0] & 0xffffffff, dat[1] >> 32, dat[1] & 0xffffffff.
 * <prefix>.oc  ovFileOCW (src/stores/ovStoreFile.H:50-115): uint64 number of records,
 *              uint32 oprMax = last read ID + 1, uint32 opr[oprMax] = records naming each
 *              read as a or b.
 *
 * The .oc prefix is the .ovb name cut at the first '.' of its last path component:
 * canu runs `overlapInCore -o ./<job>.ovb.WORKING` and collects ./<job>.oc
 * (src/pipelines/canu/OverlapInCore.pm:187-197).
 *
 * Every function returns 0 on success, 1 on a failed open/read/write/close (errno is
 * left set), 2 on a malformed file or argument.
 */
#ifndef OIC_OVFILE_H
#define OIC_OVFILE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Words per .ovb block (ovStoreFile.C:112-121 with the default 1 MiB buffer). */
#define OIC_OVB_BLOCK_WORDS 262080u

/* Write nRecords records (6 uint32 words each) to path.  framing 1: snappy blocks as
 * ovFile::writeBuffer writes them (ovStoreFile.C:224-238), compressed with the
 * library's own snappy encoder; framing 0: the words unframed.  The file is written
 * completely or the call fails (a short write or a failed close returns 1). */
int oic_ovb_write(const char *path, const uint32_t *words, uint64_t nRecords, int framing);

/* Read a snappy-framed .ovb (ovFile::loadBuffer / readOverlap, ovStoreFile.C:327-399).
 * With words NULL only counts: *nRecords gets the number of records.  Otherwise copies
 * up to maxRecords records; a file holding more returns 2 after filling words. */
int oic_ovb_read(const char *path, uint32_t *words, uint64_t maxRecords, uint64_t *nRecords);

/* The .oc name for an .ovb name (see above) into out (capacity cap bytes). */
int oic_oc_path(const char *ovbPath, char *out, size_t cap);

/* Write the .oc counts of nRecords records for a store whose last read ID is lastID. */
int oic_oc_write(const char *path, const uint32_t *words, uint64_t nRecords, uint32_t lastID);

/* Read an .oc file: *nOlaps, and up to maxReads + 1 per-read counts into opr (NULL:
 * only the header); *oprMax gets the array length in the file. */
int oic_oc_read(const char *path, uint64_t *nOlaps, uint32_t *opr, uint32_t maxReads, uint32_t *oprMax);

/* Merge the outputs of independent jobs (hash-block x ref-range partitions of one
 * store, src/overlapInCore/overlapInCorePartition.C:225-245) into one output: the .ovb
 * blocks of inputs[0..n) are copied in order into outOvb (each block is independent),
 * and their .oc files are summed into outOvb's .oc. */
int oic_merge_outputs(const char *outOvb, const char *const *inputs, uint32_t n);

/* Records per data file of an overlap store (OVFILE_MAX_OVERLAPS, src/stores/
 * ovStoreFile.H:27: 1 GiB of 20-byte records). */
#define OIC_OVSTORE_MAX_PER_FILE 53687091u

/* Write an overlap-store directory as canu's sequential store writer lays it out
 * (ovStoreWriter, src/stores/ovStoreWriter.C:25-130), the last step of ovStoreBuild
 * (src/stores/ovStoreBuild.C:255-270), so that canu's ovStore reader
 * (src/stores/ovStore.C) opens it:
 *   dir/info        ovStoreInfo (ovStore.H:39-137): uint64 magic "canu:OVS", uint64
 *                   version 4, uint32 read-length bits (21), uint32 first and last read
 *                   ID with overlaps, uint32 maxID, uint64 records;
 *   dir/index       ovStoreOfft (ovStore.H:140-170) per read ID 0..maxID: uint16 slice
 *                   (1), uint16 data file, uint32 position of the read's first record in
 *                   that file, uint32 records, 4 zero bytes, uint64 index of the read's
 *                   first record in the store;
 *   dir/0001-NNN    the data files: five uint32 words per record (the record without
 *                   a_iid); a new file starts at a read's first record once the current
 *                   one holds more than maxPerFile records (0: OIC_OVSTORE_MAX_PER_FILE);
 *   dir/statistics  (only with records) uint32 maxID, 0, maxID, then per read ID 0..maxID
 *                   16 uint16 ranks and 16 uint16 scores sampled from its overlaps' scores
 *                   sorted decreasing (ovStoreHistogram.C:135-259, the overlap score of
 *                   ovOverlap.H:243-247).
 * rec: nRecords store records (six words: a_iid, b_iid, dat[0] >> 32, dat[0] & 0xffffffff,
 * dat[1] >> 32, dat[1] & 0xffffffff) sorted as oic_store_sort returns them; readLen[i]: the
 * length of read ID i+1, i < maxID.  Returns 2 for records out of order, IDs outside
 * 1..maxID, A hangs longer than the A read or maxPerFile above 2^31 - 1 (the index holds
 * 32-bit offsets); 1 when a file cannot be written (files already written stay). */
int oic_ovstore_write(const char *dir, const uint32_t *rec, uint64_t nRecords, const uint32_t *readLen,
                      uint32_t maxID, uint64_t maxPerFile);

/* Raw snappy block of src[0..n) into dst (capacity at least oic_snappy_max_length(n));
 * *dstLen gets its length.  The block decodes with any snappy decoder. */
size_t oic_snappy_max_length(size_t n);
int    oic_snappy_compress(const uint8_t *src, size_t n, uint8_t *dst, size_t *dstLen);
/* Decode a raw snappy block (cap: bytes available at dst). */
int    oic_snappy_uncompress(const uint8_t *src, size_t n, uint8_t *dst, size_t cap, size_t *dstLen);

#ifdef __cplusplus
}
#endif

#endif
