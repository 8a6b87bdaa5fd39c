// cr_potree.cpp -- Potree 2.0 octrees into the batched layout
// (include/cr_potree.h; the reference's PotreeData, modules/compute/PotreeData.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cr_potree.h"
#include "cr_internal.h"

namespace {

// ---- a small JSON reader: objects, arrays, numbers, strings, literals -------

struct Json {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    double num = 0.0;
    bool b = false;
    std::string str;
    std::vector<Json> items;
    std::vector<std::pair<std::string, Json>> members;

    const Json* get(const char* key) const {
        if (kind != Object) return nullptr;
        for (const auto& m : members)
            if (m.first == key) return &m.second;
        return nullptr;
    }
};

class JsonParser {
  public:
    explicit JsonParser(const std::string& s) : s_(s) {}
    bool parse(Json* out) {
        if (!value(out, 0)) return false;
        ws();
        return i_ == s_.size();
    }

  private:
    const std::string& s_;
    size_t i_ = 0;

    void ws() {
        while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\t' || s_[i_] == '\n' || s_[i_] == '\r')) i_++;
    }
    bool lit(const char* w) {
        const size_t n = std::strlen(w);
        if (s_.compare(i_, n, w) != 0) return false;
        i_ += n;
        return true;
    }
    bool string(std::string* out) {
        if (i_ >= s_.size() || s_[i_] != '"') return false;
        i_++;
        while (i_ < s_.size() && s_[i_] != '"') {
            char c = s_[i_++];
            if (c == '\\') {
                if (i_ >= s_.size()) return false;
                const char e = s_[i_++];
                switch (e) {
                    case 'n': c = '\n'; break;
                    case 't': c = '\t'; break;
                    case 'r': c = '\r'; break;
                    case 'b': c = '\b'; break;
                    case 'f': c = '\f'; break;
                    case 'u':  // names and values here are ASCII; keep the escape as '?'
                        if (i_ + 4 > s_.size()) return false;
                        i_ += 4;
                        c = '?';
                        break;
                    default: c = e;
                }
            }
            out->push_back(c);
        }
        if (i_ >= s_.size()) return false;
        i_++;
        return true;
    }
    bool value(Json* v, int depth) {
        if (depth > 64) return false;
        ws();
        if (i_ >= s_.size()) return false;
        const char c = s_[i_];
        if (c == '{') {
            v->kind = Json::Object;
            i_++;
            ws();
            if (i_ < s_.size() && s_[i_] == '}') return ++i_, true;
            while (true) {
                ws();
                std::string key;
                if (!string(&key)) return false;
                ws();
                if (i_ >= s_.size() || s_[i_] != ':') return false;
                i_++;
                Json m;
                if (!value(&m, depth + 1)) return false;
                v->members.emplace_back(std::move(key), std::move(m));
                ws();
                if (i_ < s_.size() && s_[i_] == ',') { i_++; continue; }
                if (i_ < s_.size() && s_[i_] == '}') return ++i_, true;
                return false;
            }
        }
        if (c == '[') {
            v->kind = Json::Array;
            i_++;
            ws();
            if (i_ < s_.size() && s_[i_] == ']') return ++i_, true;
            while (true) {
                Json m;
                if (!value(&m, depth + 1)) return false;
                v->items.push_back(std::move(m));
                ws();
                if (i_ < s_.size() && s_[i_] == ',') { i_++; continue; }
                if (i_ < s_.size() && s_[i_] == ']') return ++i_, true;
                return false;
            }
        }
        if (c == '"') {
            v->kind = Json::String;
            return string(&v->str);
        }
        if (lit("true")) { v->kind = Json::Bool; v->b = true; return true; }
        if (lit("false")) { v->kind = Json::Bool; v->b = false; return true; }
        if (lit("null")) { v->kind = Json::Null; return true; }
        // number: the C library's strtod on the token
        const size_t start = i_;
        while (i_ < s_.size() && (std::strchr("+-0123456789.eE", s_[i_]) != nullptr)) i_++;
        if (i_ == start) return false;
        const std::string tok = s_.substr(start, i_ - start);
        char* end = nullptr;
        v->kind = Json::Number;
        v->num = std::strtod(tok.c_str(), &end);
        return end && *end == '\0';
    }
};

bool num(const Json* j, double* out) {
    if (!j || j->kind != Json::Number) return false;
    *out = j->num;
    return true;
}

bool vec3(const Json* j, double out[3]) {
    if (!j || j->kind != Json::Array || j->items.size() != 3) return false;
    for (int k = 0; k < 3; k++)
        if (!num(&j->items[k], &out[k])) return false;
    return true;
}

bool read_file(const std::string& path, std::string* out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    *out = ss.str();
    return true;
}

// ---- the octree ---------------------------------------------------------------

struct Node {
    int level = 0;
    int type = 0;
    int child_mask = 0;
    int64_t num_points = 0, byte_offset = 0, byte_size = 0;
    int64_t hier_offset = 0, hier_size = 0;
    double min[3] = {0, 0, 0}, max[3] = {0, 0, 0};
    int children[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
};

// PotreeData.h:112-140 createChildAABB: the parent's box converted to float,
// halved in float arithmetic per axis (bit 0: z, bit 1: y, bit 2: x).
void child_box(const Node& parent, int index, Node* child) {
    float mn[3], mx[3], size[3];
    for (int k = 0; k < 3; k++) {
        mn[k] = (float)parent.min[k];
        mx[k] = (float)parent.max[k];
        size[k] = mx[k] - mn[k];
    }
    const int axis_bit[3] = {4, 2, 1};  // x, y, z
    for (int k = 0; k < 3; k++) {
        if (index & axis_bit[k]) mn[k] = mn[k] + size[k] / 2.0f;
        else mx[k] = mx[k] - size[k] / 2.0f;
    }
    for (int k = 0; k < 3; k++) {
        child->min[k] = mn[k];
        child->max[k] = mx[k];
    }
}

int64_t rd_i64(const std::string& b, size_t o) { int64_t v; std::memcpy(&v, b.data() + o, 8); return v; }
uint32_t rd_u32(const std::string& b, size_t o) { uint32_t v; std::memcpy(&v, b.data() + o, 4); return v; }

}  // namespace

struct cr_potree {
    cr_potree_info info{};
    std::string dir;
    std::vector<Node> nodes;  // sorted by byte_offset
};

namespace {

constexpr int kEntryBytes = 22;  // PotreeData.h:188

// PotreeData.h:186-258 parseHierarchy: the chunk at the proxy's
// [hier_offset, hier_offset + hier_size) lists its nodes breadth first, the
// chunk's root first; children are created in child-index order; proxy
// entries (type 2) defer their subtree to another chunk.
bool parse_chunk(std::vector<Node>& all, int root, const std::string& buf, int depth) {
    if (depth > 64) return false;
    const Node r = all[root];
    if (r.hier_size % kEntryBytes != 0 || r.hier_offset < 0 ||
        r.hier_offset + r.hier_size > (int64_t)buf.size())
        return false;
    const int64_t n = r.hier_size / kEntryBytes;
    std::vector<int> order;
    order.reserve((size_t)n);
    order.push_back(root);
    std::vector<int> proxies;
    for (int64_t i = 0; i < n; i++) {
        if (i >= (int64_t)order.size()) return false;  // fewer nodes than entries
        const int cur = order[(size_t)i];
        const size_t o = (size_t)(r.hier_offset + i * kEntryBytes);
        const int type = (uint8_t)buf[o];
        const int mask = (uint8_t)buf[o + 1];
        const int64_t np = rd_u32(buf, o + 2);
        const int64_t off = rd_i64(buf, o + 6), size = rd_i64(buf, o + 14);
        {
            Node& c = all[cur];
            if (c.type == 2) {  // a chunk's root, until now the proxy its parent listed
                c.byte_offset = off;
                c.byte_size = size;
            } else if (type == 2) {
                c.hier_offset = off;
                c.hier_size = size;
            } else {
                c.byte_offset = off;
                c.byte_size = size;
            }
            c.num_points = np;
            c.type = type;
            c.child_mask = mask;
        }
        if (type == 2) {
            proxies.push_back(cur);
            continue;
        }
        for (int ci = 0; ci < 8; ci++) {
            if (!((mask >> ci) & 1)) continue;
            Node child;
            child_box(all[cur], ci, &child);
            child.level = all[cur].level + 1;
            all.push_back(child);
            const int id = (int)all.size() - 1;
            all[cur].children[ci] = id;
            order.push_back(id);
        }
    }
    for (int p : proxies)
        if (!parse_chunk(all, p, buf, depth + 1)) return false;
    return true;
}

void preorder(const std::vector<Node>& all, int id, std::vector<Node>* out) {
    out->push_back(all[id]);
    for (int c : all[id].children)
        if (c >= 0) preorder(all, c, out);
}

// uint32(t) & MASK_30BIT (PotreeData.h:420-422), or a clamp to [0, 2^30 - 1].
// A double below zero converts as the x86-64 compilers the reference builds
// with do (through a 64-bit integer); NaN (a zero extent) gives 0.
uint32_t quantize(double t, bool wrap) {
    if (t != t) return 0u;
    if (wrap) {
        const double c = t < -9.0e18 ? -9.0e18 : (t > 9.0e18 ? 9.0e18 : t);
        return (uint32_t)(int64_t)c & 1073741823u;
    }
    if (!(t > 0.0)) return 0u;
    return t >= 1073741823.0 ? 1073741823u : (uint32_t)t;
}

}  // namespace

extern "C" {

cr_status cr_potree_open(const char* dir, cr_potree** out, cr_potree_info* info) {
    if (!dir || !out) return CR_ERR_INVALID_ARG;
    *out = nullptr;
    std::string text, hier;
    const std::string d(dir);
    if (!read_file(d + "/metadata.json", &text) || !read_file(d + "/hierarchy.bin", &hier))
        return CR_ERR_NOT_FOUND;
    Json js;
    if (!JsonParser(text).parse(&js) || js.kind != Json::Object) return CR_ERR_INVALID_ARG;
    std::unique_ptr<cr_potree> p(new (std::nothrow) cr_potree());
    if (!p) return CR_ERR_OUT_OF_MEMORY;
    cr_potree_info& in = p->info;
    double points = 0, first_chunk = 0;
    const Json* bb = js.get("boundingBox");
    const Json* h = js.get("hierarchy");
    if (!bb || !vec3(bb->get("min"), in.box_min) || !vec3(bb->get("max"), in.box_max) ||
        !vec3(js.get("scale"), in.scale) || !vec3(js.get("offset"), in.offset) ||
        !num(js.get("points"), &points) || !num(js.get("spacing"), &in.spacing) || !h ||
        !num(h->get("firstChunkSize"), &first_chunk))
        return CR_ERR_INVALID_ARG;
    const Json* enc = js.get("encoding");
    if (enc && enc->kind == Json::String && enc->str != "DEFAULT") return CR_ERR_UNSUPPORTED;
    in.num_points = (int64_t)points;
    // PotreeData.h:171-182: the point record is the attributes back to back
    const Json* attrs = js.get("attributes");
    if (!attrs || attrs->kind != Json::Array) return CR_ERR_INVALID_ARG;
    in.rgb_offset = -1;
    int64_t bpp = 0;
    for (const Json& a : attrs->items) {
        const Json* name = a.get("name");
        double size = 0;
        if (!name || name->kind != Json::String || !num(a.get("size"), &size) || size < 0)
            return CR_ERR_INVALID_ARG;
        if (name->str == "rgb") in.rgb_offset = (int32_t)bpp;
        bpp += (int64_t)size;
    }
    if (bpp < 12 || bpp > 4096 || in.num_points < 0 || in.num_points >= ((int64_t)1 << 31) - 64 ||
        (in.rgb_offset >= 0 && in.rgb_offset + 6 > bpp))
        return CR_ERR_INVALID_ARG;
    in.bytes_per_point = (int32_t)bpp;

    // PotreeData.h:260-315 loadHierarchy: the root box is (0, 0, 0) to
    // boxMax - boxMin, its first chunk firstChunkSize bytes at offset 0
    std::vector<Node> all(1);
    all[0].type = 2;
    all[0].hier_offset = 0;
    all[0].hier_size = (int64_t)first_chunk;
    for (int k = 0; k < 3; k++) all[0].max[k] = in.box_max[k] - in.box_min[k];
    if (!parse_chunk(all, 0, hier, 0)) return CR_ERR_INVALID_ARG;
    std::vector<Node> nodes;
    preorder(all, 0, &nodes);
    std::stable_sort(nodes.begin(), nodes.end(),
                     [](const Node& a, const Node& b) { return a.byte_offset < b.byte_offset; });
    in.num_nodes = (int64_t)nodes.size();
    for (const Node& n : nodes) {
        if (n.num_points < 0 || n.byte_offset < 0 || n.byte_offset % bpp != 0 ||
            n.byte_offset / bpp + n.num_points > in.num_points)
            return CR_ERR_INVALID_ARG;
        in.max_level = std::max(in.max_level, n.level);
        in.max_node_points = std::max(in.max_node_points, n.num_points);
        in.octree_bytes = std::max(in.octree_bytes, n.byte_offset + n.num_points * bpp);
    }
    if (in.num_nodes >= cr::kMaxBatches) return CR_ERR_INVALID_ARG;
    p->nodes = std::move(nodes);
    p->dir = d;
    if (info) *info = in;
    *out = p.release();
    return CR_OK;
}

cr_status cr_potree_close(cr_potree* p) {
    if (!p) return CR_ERR_INVALID_ARG;
    delete p;
    return CR_OK;
}

cr_status cr_potree_nodes(const cr_potree* p, cr_potree_node* out, int64_t max) {
    if (!p || (!out && max > 0) || max < (int64_t)p->nodes.size()) return CR_ERR_INVALID_ARG;
    for (size_t i = 0; i < p->nodes.size(); i++) {
        const Node& n = p->nodes[i];
        cr_potree_node& o = out[i];
        std::memset(&o, 0, sizeof(o));
        o.level = n.level;
        o.type = n.type;
        o.child_mask = n.child_mask;
        o.num_points = n.num_points;
        o.byte_offset = n.byte_offset;
        o.byte_size = n.byte_size;
        for (int k = 0; k < 3; k++) {
            o.min[k] = n.min[k];
            o.max[k] = n.max[k];
        }
    }
    return CR_OK;
}

// PotreeData.h:335-350 (batch records) and :361-452 (the loader thread's
// per-point encoding), for every node at once.
cr_status cr_potree_encode(const cr_potree* p, const uint8_t* octree, int64_t bytes, int32_t quirks,
                           cr_batch* batches, uint32_t* lo, uint32_t* md, uint32_t* hi,
                           uint32_t* rgba) {
    if (!p || (!octree && bytes > 0) || bytes < p->info.octree_bytes || !batches || !lo || !md ||
        !hi || !rgba)
        return CR_ERR_INVALID_ARG;
    const int q = quirks == CR_POTREE_QUIRKS_DEFAULT ? (CR_POTREE_QUIRK_12B_FROM_8B | CR_POTREE_QUIRK_WRAP30)
                                                     : quirks;
    const bool wrap = (q & CR_POTREE_QUIRK_WRAP30) != 0, x12_from_8 = (q & CR_POTREE_QUIRK_12B_FROM_8B) != 0;
    const cr_potree_info& in = p->info;
    const int64_t bpp = in.bytes_per_point;
    const double steps = 1073741824.0;
    for (int64_t i = 0; i < in.num_points; i++) lo[i] = md[i] = hi[i] = rgba[i] = 0u;
    for (size_t i = 0; i < p->nodes.size(); i++) {
        const Node& n = p->nodes[i];
        cr_batch& b = batches[i];
        std::memset(&b, 0, sizeof(b));
        b.min_x = (float)n.min[0]; b.min_y = (float)n.min[1]; b.min_z = (float)n.min[2];
        b.max_x = (float)n.max[0]; b.max_y = (float)n.max[1]; b.max_z = (float)n.max[2];
        b.num_points = (int32_t)std::min<int64_t>(n.num_points, INT32_MAX);
        b.first_point = (int32_t)(n.byte_offset / bpp);
        b.file_index = n.level;  // the Batch's `level` (compute_loop_nodes/render.cs:28-45)
        const double size[3] = {n.max[0] - n.min[0], n.max[1] - n.min[1], n.max[2] - n.min[2]};
        for (int64_t j = 0; j < n.num_points; j++) {
            const int64_t pi = n.byte_offset / bpp + j;
            const uint8_t* r = octree + pi * bpp;
            uint32_t Q[3];
            for (int k = 0; k < 3; k++) {
                int32_t X;
                std::memcpy(&X, r + 4 * k, 4);
                const double x = (double)X * in.scale[k] + in.offset[k] - in.box_min[k];
                Q[k] = quantize(((x - n.min[k]) / size[k]) * steps, wrap);
            }
            auto word = [&](int shift) {
                return ((Q[0] >> shift) & 1023u) | (((Q[1] >> shift) & 1023u) << 10) |
                       (((Q[2] >> shift) & 1023u) << 20);
            };
            lo[pi] = word(20);
            md[pi] = word(10);
            hi[pi] = x12_from_8 ? word(10) : word(0);
            uint32_t c = 0;
            if (in.rgb_offset >= 0) {
                uint32_t ch[3];
                for (int k = 0; k < 3; k++) {
                    uint16_t v;
                    std::memcpy(&v, r + in.rgb_offset + 2 * k, 2);
                    ch[k] = v > 255 ? v / 256u : v;
                }
                c = ch[0] | (ch[1] << 8) | (ch[2] << 16);
            }
            rgba[pi] = c;
        }
    }
    return CR_OK;
}

cr_status cr_potree_load(cr_ctx* ctx, const cr_potree* p, int32_t quirks, cr_cloud** out,
                         void* stream) {
    if (!ctx || !p || !out) return CR_ERR_INVALID_ARG;
    *out = nullptr;
    std::ifstream f(p->dir + "/octree.bin", std::ios::binary);
    if (!f) return CR_ERR_NOT_FOUND;
    const int64_t bytes = p->info.octree_bytes;
    std::vector<uint8_t> oct((size_t)std::max<int64_t>(bytes, 1));
    if (bytes > 0 && !f.read(reinterpret_cast<char*>(oct.data()), bytes)) return CR_ERR_INVALID_ARG;
    const int64_t n = p->info.num_points, nb = p->info.num_nodes;
    std::vector<cr_batch> batches((size_t)nb);
    std::vector<uint32_t> lo((size_t)n), md((size_t)n), hi((size_t)n), rgba((size_t)n);
    cr_status s = cr_potree_encode(p, oct.data(), bytes, quirks, batches.data(), lo.data(), md.data(),
                                   hi.data(), rgba.data());
    if (s != CR_OK) return s;
    cr_cloud* c = nullptr;
    s = cr_cloud_create(ctx, n, nb, 1, CR_STREAM_ALL, &c);
    if (s != CR_OK) return s;
    const double origin[3] = {0.0, 0.0, 0.0};
    // the records carry the node level in file_index; loop_nodes renders every
    // node with the one world matrix (CR_QUIRK_ONE_WORLD), so they go in
    // without the per-file check cr_cloud_upload applies to records
    cr_batch* db = nullptr;
    s = cr_cloud_device(c, &db, nullptr, nullptr, nullptr, nullptr);
    if (s == CR_OK)
        s = cr_cloud_upload(ctx, c, nullptr, lo.data(), md.data(), hi.data(), rgba.data(), origin, stream);
    if (s == CR_OK && nb > 0 &&
        cudaMemcpyAsync(db, batches.data(), sizeof(cr_batch) * (size_t)nb, cudaMemcpyHostToDevice,
                        (cudaStream_t)stream) != cudaSuccess)
        s = CR_ERR_CUDA;
    if (s == CR_OK && cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) s = CR_ERR_CUDA;
    if (s != CR_OK) {
        cr_cloud_destroy(ctx, c);
        return s;
    }
    *out = c;
    return CR_OK;
}

}  // extern "C"
