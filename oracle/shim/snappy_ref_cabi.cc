// snappy_ref_cabi.cc -- C entry points over the snappy sources vendored in canu's tree
// (src/stores/libsnappy), for the tests (ctypes).  Test infrastructure only: the tests
// decode the engine's .ovb blocks with the same snappy code canu's ovFile reader runs
// (src/stores/ovStoreFile.C:341-372), and compress with the code its writer runs
// (src/stores/ovStoreFile.C:224-238).
#include <cstddef>

#include "snappy.h"

extern "C" {

int snappy_ref_uncompressed_length(const char *src, size_t n, size_t *len) {
  return snappy::GetUncompressedLength(src, n, len) ? 0 : 1;
}

int snappy_ref_uncompress(const char *src, size_t n, char *dst) { return snappy::RawUncompress(src, n, dst) ? 0 : 1; }

int snappy_ref_is_valid(const char *src, size_t n) { return snappy::IsValidCompressedBuffer(src, n) ? 1 : 0; }

size_t snappy_ref_max_compressed_length(size_t n) { return snappy::MaxCompressedLength(n); }

void snappy_ref_compress(const char *src, size_t n, char *dst, size_t *len) { snappy::RawCompress(src, n, dst, len); }
}
