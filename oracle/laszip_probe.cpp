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

// Per-item buffers in LASzip's in-memory item layout.  LASzip's raw item
// readers and writers convert LAS records to and from that layout; for LAS 1.4
// points the layout's extended_point_type bits (byte 22) must be set, as the
// LASzip DLL sets them for point formats 6-10.
struct Items {
    std::vector<std::vector<U8>> buf;
    std::vector<U8*> ptr;
    explicit Items(const LASzip& zip) : buf(zip.num_items, std::vector<U8>(256, 0)), ptr(zip.num_items) {
        for (U32 i = 0; i < zip.num_items; i++) {
            ptr[i] = buf[i].data();
            if (zip.items[i].type == LASitem::POINT14) buf[i][22] = 1;
        }
    }
};

// item_version 4 selects LASzip's version-4 LAS 1.4 items (its fix of the
// version-3 context hand-over), which the library writes when an item asks
// for it; 0 keeps LASzip's default.
bool setup_pair(int point_format, int bytes_per_point, int compressor, uint32_t chunk_size, int item_version,
                LASzip& raw, LASzip& packed) {
    if (!raw.setup((U8)point_format, (U16)bytes_per_point, LASZIP_COMPRESSOR_NONE)) return false;
    if (!packed.setup((U8)point_format, (U16)bytes_per_point, (U16)compressor)) return false;
    if (packed.compressor != LASZIP_COMPRESSOR_POINTWISE && !packed.set_chunk_size(chunk_size)) return false;
    if (item_version == 4)
        for (U32 i = 0; i < packed.num_items; i++)
            if (packed.items[i].version == 3) packed.items[i].version = 4;
    return true;
}

}  // namespace

extern "C" {

// The LASzip VLR payload for a point type / size / compressor / chunk size.
int lzref_vlr(int point_format, int bytes_per_point, int compressor, uint32_t chunk_size,
              int item_version, uint8_t* out, int32_t cap) {
    LASzip raw, zip;
    if (!setup_pair(point_format, bytes_per_point, compressor, chunk_size, item_version, raw, zip)) return -1;
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
                       int item_version, int64_t var_every, uint8_t* out, int64_t cap) {
    LASzip raw, zip;
    if (!setup_pair(point_format, bytes_per_point, compressor, chunk_size, item_version, raw, zip)) return -1;
    LASreadPoint rr;
    if (!rr.setup(raw.num_items, raw.items)) return -1;
    ByteStreamInArrayLE rin(records, n * bytes_per_point);
    if (!rr.init(&rin)) return -1;
    LASwritePoint w;
    if (!w.setup(zip.num_items, zip.items, &zip)) return -1;
    ByteStreamOutArrayLE os;
    os.putBytes(prefix, (U32)prefix_len);
    if (!w.init(&os)) return -1;
    Items it(zip);
    for (int64_t i = 0; i < n; i++) {
        if (chunk_size == 0xFFFFFFFFu && i > 0 && var_every > 0 && i % var_every == 0) w.chunk();
        if (!rr.read(it.ptr.data())) return -1;
        if (!w.write(it.ptr.data())) return -1;
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
    U8 point_type = 0;
    U16 record_length = 0;
    if (!zip.is_standard(&point_type, &record_length)) return -1;
    LASzip raw;
    if (!raw.setup(point_type, record_length, LASZIP_COMPRESSOR_NONE)) return -1;
    LASreadPoint r;
    if (!r.setup(zip.num_items, zip.items, &zip)) return -1;
    ByteStreamInArrayLE is(file, size);
    if (!is.seek(points_at)) return -1;
    if (!r.init(&is)) return -1;
    LASwritePoint wr;
    if (!wr.setup(raw.num_items, raw.items)) return -1;
    ByteStreamOutArrayLE os;
    if (!wr.init(&os)) return -1;
    Items it(zip);
    int64_t i = 0;
    for (; i < n; i++) {
        if (!r.read(it.ptr.data())) break;
        if (!wr.write(it.ptr.data())) return -1;
    }
    r.done();
    std::memcpy(records, os.getData(), (size_t)os.getSize());
    (void)bytes_per_point;
    return i;
}

}  // extern "C"
