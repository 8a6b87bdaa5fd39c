// laszip_probe.cpp -- TEST INFRASTRUCTURE.  Compiled by oracle/Makefile
// against the reference's vendored LASzip sources (libs/laszip/src: the
// arithmetic coder, integer compressor, item codecs v1-v4 and the point
// reader / writer; not laszip_dll.cpp, whose API header is generated by its
// CMake build) into oracle/_ref/liblaszipref.so.  The CPU tests use it to
// write .laz fixtures with LASzip's own compressor and to check the product's
// decoder and writer against LASzip byte for byte.
#include <cstdint>
#include <cstring>
#include <vector>

#include "bytestreamin_array.hpp"
#include "bytestreamout_array.hpp"
#include "lasreadpoint.hpp"
#include "laswritepoint.hpp"
#include "laszip.hpp"

namespace {

// Item pointers into one record, in the item order of the LASzip setup.
void item_pointers(const LASzip& zip, U8* rec, std::vector<U8*>& ptrs) {
    ptrs.resize(zip.num_items);
    U32 off = 0;
    for (U32 i = 0; i < zip.num_items; i++) {
        ptrs[i] = rec + off;
        off += zip.items[i].size;
    }
}

}  // namespace

extern "C" {

// The LASzip VLR payload for a point type / size / compressor / chunk size.
int lzref_vlr(int point_format, int bytes_per_point, int compressor, uint32_t chunk_size,
              uint8_t* out, int32_t cap) {
    LASzip zip;
    if (!zip.setup((U8)point_format, (U16)bytes_per_point, (U16)compressor)) return -1;
    if (compressor >= LASZIP_COMPRESSOR_POINTWISE_CHUNKED && !zip.set_chunk_size(chunk_size)) return -1;
    U8* bytes = nullptr;
    I32 num = 0;
    if (!zip.pack(bytes, num) || num > cap) return -1;
    std::memcpy(out, bytes, num);
    return num;
}

// Writes `prefix` (LAS header and VLRs) and the compressed points; with a
// chunk size of 0xFFFFFFFF a chunk is closed after every `var_every` points.
int64_t lzref_compress(const uint8_t* prefix, int64_t prefix_len, const uint8_t* records, int64_t n,
                       int point_format, int bytes_per_point, int compressor, uint32_t chunk_size,
                       int64_t var_every, uint8_t* out, int64_t cap) {
    LASzip zip;
    if (!zip.setup((U8)point_format, (U16)bytes_per_point, (U16)compressor)) return -1;
    if (compressor >= LASZIP_COMPRESSOR_POINTWISE_CHUNKED && !zip.set_chunk_size(chunk_size)) return -1;
    LASwritePoint w;
    if (!w.setup(zip.num_items, zip.items, &zip)) return -1;
    ByteStreamOutArrayLE os;
    os.putBytes(prefix, (U32)prefix_len);
    if (!w.init(&os)) return -1;
    std::vector<U8> rec(bytes_per_point);
    std::vector<U8*> ptrs;
    item_pointers(zip, rec.data(), ptrs);
    for (int64_t i = 0; i < n; i++) {
        if (chunk_size == 0xFFFFFFFFu && i > 0 && var_every > 0 && i % var_every == 0) w.chunk();
        std::memcpy(rec.data(), records + i * bytes_per_point, bytes_per_point);
        if (!w.write(ptrs.data())) return -1;
    }
    if (!w.done()) return -1;
    const int64_t size = os.getSize();
    if (size > cap) return -size;
    std::memcpy(out, os.getData(), size);
    return size;
}

// Decompresses n points starting at `points_at` (the offset to point data),
// with the VLR payload `vlr`, into records.  Returns the points read.
int64_t lzref_decompress(const uint8_t* file, int64_t size, int64_t points_at, const uint8_t* vlr,
                         int32_t vlr_len, int64_t n, int bytes_per_point, uint8_t* records) {
    LASzip zip;
    if (!zip.unpack(vlr, vlr_len)) return -1;
    LASreadPoint r;
    if (!r.setup(zip.num_items, zip.items, &zip)) return -1;
    ByteStreamInArrayLE is(file, size);
    if (!is.seek(points_at)) return -1;
    if (!r.init(&is)) return -1;
    std::vector<U8> rec(bytes_per_point);
    std::vector<U8*> ptrs;
    item_pointers(zip, rec.data(), ptrs);
    for (int64_t i = 0; i < n; i++) {
        if (!r.read(ptrs.data())) return i;
        std::memcpy(records + i * bytes_per_point, rec.data(), bytes_per_point);
    }
    r.done();
    return n;
}

}  // extern "C"
