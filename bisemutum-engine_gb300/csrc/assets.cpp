// assets.cpp — the reference engine's on-disk formats, read into the C-ABI scene.
//
//   .static_mesh.biasset  StaticMesh::load / save (bisemutum/src/scene_basic/static_mesh.cpp:10-44):
//                         u32 magic 0x0b1a55e7 (runtime/asset.hpp:15), string type name
//                         "StaticMesh", u32 version; version 1: the MeshData byte stream;
//                         version 2: u64 length, u64 compressed length, zlib stream of it
//                         (prelude/byte_stream.cpp:28-41, 80-98).  MeshData
//                         (graphics/mesh.cpp:127-146) is eight length-prefixed arrays:
//                         positions f32x3, normals f32x3, tangents f32x4, colors f32x3,
//                         texcoords f32x2, texcoords2 f32x2, indices u32, submeshes
//                         {base_vertex, index_offset, num_indices u32, topology u8, 3 pad}.
//                         Strings and arrays carry a u64 element count.
//   TOML files            project.toml (scene_file, asset_metadata_file), asset_metadata.toml
//                         ([[assets]] id / path / type), scene.toml ([[objects]] with
//                         components, runtime/scene.cpp:103-135), material TOML
//                         (scene_basic/material.cpp:12-53).
//
// The zlib / DEFLATE decoder follows RFC 1950 / RFC 1951 (stored, fixed and
// dynamic Huffman blocks, Adler-32 check); the writer emits stored blocks, which
// any zlib decoder (the reference uses miniz's mz_uncompress) accepts.  The TOML
// reader covers what these files use: tables, arrays of tables, dotted keys,
// basic / literal / multi-line strings, integers, floats, booleans, arrays and
// inline tables.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "bsm_pt.h"

namespace {

// ================================================================ zlib ====
uint32_t adler32(const uint8_t* p, size_t n) {
    uint32_t a = 1, b = 0;
    while (n > 0) {
        size_t k = std::min<size_t>(n, 5552);  // largest run without 32-bit overflow
        n -= k;
        while (k--) { a += *p++; b += a; }
        a %= 65521u;
        b %= 65521u;
    }
    return (b << 16) | a;
}

struct Bits {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    bool bad = false;
    uint32_t get(int k) {  // k <= 24 bits, LSB first
        while (cnt < k) {
            if (pos >= n) { bad = true; return 0; }
            buf |= (uint32_t)p[pos++] << cnt;
            cnt += 8;
        }
        uint32_t v = buf & ((1u << k) - 1u);
        buf >>= k;
        cnt -= k;
        return v;
    }
    void align() { buf = 0; cnt = 0; }
};

// Canonical Huffman code: number of codes per length and symbols in code order.
struct Huff {
    uint16_t count[16];
    uint16_t sym[320];
};
// Returns false for an over-subscribed code; incomplete codes are allowed (a
// single distance code is legal).
bool huff_build(Huff& h, const uint8_t* len, int n) {
    std::memset(h.count, 0, sizeof(h.count));
    for (int i = 0; i < n; ++i) h.count[len[i]]++;
    h.count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
        left <<= 1;
        left -= h.count[l];
        if (left < 0) return false;
    }
    uint16_t off[16];
    off[1] = 0;
    for (int l = 1; l < 15; ++l) off[l + 1] = off[l] + h.count[l];
    for (int i = 0; i < n; ++i)
        if (len[i]) h.sym[off[len[i]]++] = (uint16_t)i;
    return true;
}
int huff_decode(Bits& b, const Huff& h) {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
        code |= (int)b.get(1);
        if (b.bad) return -1;
        int c = h.count[l];
        if (code - first < c) return h.sym[index + (code - first)];
        index += c;
        first += c;
        first <<= 1;
        code <<= 1;
    }
    return -1;
}

// RFC 1951 section 3.2.5: base values and extra bits of length / distance codes.
const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193,
                                257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6,
                                7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// order of the code-length code lengths in a dynamic block header
const uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

bool inflate_codes(Bits& b, std::vector<uint8_t>& out, size_t limit, const Huff& lit, const Huff& dist) {
    for (;;) {
        int s = huff_decode(b, lit);
        if (s < 0) return false;
        if (s < 256) {
            if (out.size() >= limit) return false;
            out.push_back((uint8_t)s);
        } else if (s == 256) {
            return true;
        } else {
            s -= 257;
            if (s >= 29) return false;
            size_t len = kLenBase[s] + b.get(kLenExtra[s]);
            int d = huff_decode(b, dist);
            if (d < 0 || d >= 30) return false;
            size_t back = kDistBase[d] + b.get(kDistExtra[d]);
            if (b.bad || back > out.size() || out.size() + len > limit) return false;
            size_t from = out.size() - back;
            for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);
        }
    }
}

// Raw DEFLATE stream -> bytes (at most `limit`).  `used` receives the bytes consumed.
bool inflate_raw(const uint8_t* in, size_t n, size_t limit, std::vector<uint8_t>& out, size_t* used) {
    Bits b{in, n};
    int last = 0;
    while (!last) {
        last = (int)b.get(1);
        int type = (int)b.get(2);
        if (b.bad) return false;
        if (type == 0) {
            b.align();
            if (b.pos + 4 > n) return false;
            uint32_t len = in[b.pos] | (in[b.pos + 1] << 8);
            uint32_t nlen = in[b.pos + 2] | (in[b.pos + 3] << 8);
            b.pos += 4;
            if ((len ^ 0xffffu) != nlen || b.pos + len > n || out.size() + len > limit) return false;
            out.insert(out.end(), in + b.pos, in + b.pos + len);
            b.pos += len;
        } else if (type == 1) {
            uint8_t l[320];
            int i = 0;
            for (; i < 144; ++i) l[i] = 8;
            for (; i < 256; ++i) l[i] = 9;
            for (; i < 280; ++i) l[i] = 7;
            for (; i < 288; ++i) l[i] = 8;
            Huff lit, dist;
            huff_build(lit, l, 288);
            for (i = 0; i < 30; ++i) l[i] = 5;
            huff_build(dist, l, 30);
            if (!inflate_codes(b, out, limit, lit, dist)) return false;
        } else if (type == 2) {
            int nlen = (int)b.get(5) + 257, ndist = (int)b.get(5) + 1, ncode = (int)b.get(4) + 4;
            if (b.bad || nlen > 286 || ndist > 30) return false;
            uint8_t l[320] = {0};
            for (int i = 0; i < ncode; ++i) l[kClOrder[i]] = (uint8_t)b.get(3);
            Huff cl;
            if (!huff_build(cl, l, 19)) return false;
            uint8_t lens[320] = {0};
            int i = 0;
            while (i < nlen + ndist) {
                int s = huff_decode(b, cl);
                if (s < 0) return false;
                if (s < 16) {
                    lens[i++] = (uint8_t)s;
                } else {
                    int rep = 0;
                    uint8_t v = 0;
                    if (s == 16) {
                        if (i == 0) return false;
                        v = lens[i - 1];
                        rep = 3 + (int)b.get(2);
                    } else if (s == 17) {
                        rep = 3 + (int)b.get(3);
                    } else {
                        rep = 11 + (int)b.get(7);
                    }
                    if (b.bad || i + rep > nlen + ndist) return false;
                    while (rep--) lens[i++] = v;
                }
            }
            if (lens[256] == 0) return false;
            Huff lit, dist;
            if (!huff_build(lit, lens, nlen) || !huff_build(dist, lens + nlen, ndist)) return false;
            if (!inflate_codes(b, out, limit, lit, dist)) return false;
        } else {
            return false;
        }
    }
    if (used) *used = b.pos;
    return true;
}

// zlib stream (RFC 1950) -> exactly `expect` bytes.
bool zlib_decompress(const uint8_t* in, size_t n, size_t expect, std::vector<uint8_t>& out, std::string& err) {
    if (n < 6) { err = "zlib stream too short"; return false; }
    uint8_t cmf = in[0], flg = in[1];
    if ((cmf & 0x0f) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20)) {
        err = "not a zlib stream";
        return false;
    }
    out.clear();
    out.reserve(expect);
    size_t used = 0;
    if (!inflate_raw(in + 2, n - 2, expect, out, &used)) { err = "corrupt deflate data"; return false; }
    if (out.size() != expect) { err = "decompressed length differs from the header"; return false; }
    size_t a = 2 + used;
    if (a + 4 > n) { err = "zlib stream lacks its checksum"; return false; }
    uint32_t want = ((uint32_t)in[a] << 24) | ((uint32_t)in[a + 1] << 16) | ((uint32_t)in[a + 2] << 8) | in[a + 3];
    if (want != adler32(out.data(), out.size())) { err = "zlib checksum mismatch"; return false; }
    return true;
}

// bytes -> zlib stream of stored blocks.
std::vector<uint8_t> zlib_store(const uint8_t* p, size_t n) {
    std::vector<uint8_t> z = {0x78, 0x01};
    size_t off = 0;
    do {
        size_t k = std::min<size_t>(n - off, 65535);
        z.push_back(off + k == n ? 1 : 0);
        z.push_back((uint8_t)(k & 0xff));
        z.push_back((uint8_t)(k >> 8));
        z.push_back((uint8_t)(~k & 0xff));
        z.push_back((uint8_t)((~k >> 8) & 0xff));
        z.insert(z.end(), p + off, p + off + k);
        off += k;
    } while (off < n);
    uint32_t a = adler32(p, n);
    for (int s = 24; s >= 0; s -= 8) z.push_back((uint8_t)(a >> s));
    return z;
}

// ======================================================== byte streams ====
struct Reader {
    const uint8_t* p;
    size_t n, pos = 0;
    bool ok = true;
    bool raw(void* dst, size_t k) {
        if (!ok || k > n - pos) { ok = false; return false; }
        std::memcpy(dst, p + pos, k);
        pos += k;
        return true;
    }
    template <typename T> T get() { T v{}; raw(&v, sizeof(T)); return v; }
    std::string str() {
        uint64_t k = get<uint64_t>();
        if (!ok || k > n - pos) { ok = false; return {}; }
        std::string s((const char*)p + pos, (size_t)k);
        pos += (size_t)k;
        return s;
    }
    // a u64 element count followed by count * elem bytes
    template <typename T> std::vector<T> vec(size_t elem = sizeof(T)) {
        uint64_t k = get<uint64_t>();
        std::vector<T> v;
        if (!ok || elem == 0 || k > (n - pos) / elem) { ok = false; return v; }
        v.resize((size_t)k);
        raw(v.data(), (size_t)k * elem);
        return v;
    }
};

struct Writer {
    std::vector<uint8_t> b;
    void raw(const void* p, size_t k) { b.insert(b.end(), (const uint8_t*)p, (const uint8_t*)p + k); }
    template <typename T> void put(T v) { raw(&v, sizeof(T)); }
    void str(const std::string& s) { put<uint64_t>(s.size()); raw(s.data(), s.size()); }
    void arr(const void* p, uint64_t count, size_t elem) { put<uint64_t>(count); if (count) raw(p, (size_t)count * elem); }
};

const uint32_t kAssetMagic = 0x0b1a55e7u;
const char* kMeshType = "StaticMesh";

struct SubmeshRaw {  // SubmeshDesc as stored: three u32, topology u8, 3 bytes of padding
    uint32_t base_vertex, index_offset, num_indices;
    uint8_t topology, pad[3];
};
static_assert(sizeof(SubmeshRaw) == 16, "SubmeshDesc layout");

struct MeshOwned {
    std::vector<float> pos, nrm, tan, col, uv, uv2;
    std::vector<uint32_t> idx;
    std::vector<bsm_submesh> sub;
};

// Reads MeshData (mesh.cpp:137-146) into `m`.
bool read_mesh_arrays(Reader& r, MeshOwned& m) {
    auto arr = [&](std::vector<float>& dst, int comps) {
        uint64_t k = r.get<uint64_t>();
        if (!r.ok || k > (r.n - r.pos) / (4u * comps)) { r.ok = false; return; }
        dst.resize((size_t)k * comps);
        r.raw(dst.data(), dst.size() * 4);
    };
    arr(m.pos, 3);
    arr(m.nrm, 3);
    arr(m.tan, 4);
    arr(m.col, 3);
    arr(m.uv, 2);
    arr(m.uv2, 2);
    m.idx = r.vec<uint32_t>();
    std::vector<SubmeshRaw> sub = r.vec<SubmeshRaw>();
    if (!r.ok) return false;
    m.sub.resize(sub.size());
    for (size_t i = 0; i < sub.size(); ++i)
        m.sub[i] = bsm_submesh{sub[i].base_vertex, sub[i].index_offset, sub[i].num_indices, sub[i].topology};
    return true;
}

bool read_static_mesh(const uint8_t* p, size_t n, MeshOwned& m, std::string& err) {
    Reader r{p, n};
    uint32_t magic = r.get<uint32_t>();
    std::string type = r.str();
    uint32_t version = r.get<uint32_t>();
    if (!r.ok || magic != kAssetMagic) { err = "not a bisemutum binary asset (bad magic)"; return false; }
    if (type != kMeshType) { err = "asset type is '" + type + "', not StaticMesh"; return false; }
    if (version == 1) {
        if (!read_mesh_arrays(r, m)) { err = "truncated mesh data"; return false; }
        return true;
    }
    if (version != 2) { err = "unknown StaticMesh version " + std::to_string(version); return false; }
    uint64_t len = r.get<uint64_t>();
    uint64_t clen = r.get<uint64_t>();
    if (!r.ok || clen > n - r.pos || len > (1ull << 34)) { err = "truncated compressed part"; return false; }
    std::vector<uint8_t> raw;
    if (!zlib_decompress(p + r.pos, (size_t)clen, (size_t)len, raw, err)) return false;
    Reader d{raw.data(), raw.size()};
    if (!read_mesh_arrays(d, m)) { err = "truncated mesh data"; return false; }
    return true;
}

// ================================================================ TOML ====
struct TVal {
    enum Kind { None, Str, Int, Float, Bool, Arr, Tab } k = None;
    std::string s;
    int64_t i = 0;
    double f = 0.0;
    bool b = false;
    std::vector<TVal> a;
    std::vector<std::pair<std::string, TVal>> t;

    const TVal* get(const std::string& key) const {
        if (k != Tab) return nullptr;
        for (auto& kv : t)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    TVal* slot(const std::string& key) {
        for (auto& kv : t)
            if (kv.first == key) return &kv.second;
        t.emplace_back(key, TVal{});
        return &t.back().second;
    }
    bool is_num() const { return k == Int || k == Float; }
    double num() const { return k == Int ? (double)i : f; }
};

double num_or(const TVal* v, double d) { return v && v->is_num() ? v->num() : d; }
bool vec_of(const TVal* v, int n, double* out) {
    if (!v || v->k != TVal::Arr || (int)v->a.size() != n) return false;
    for (int c = 0; c < n; ++c) {
        if (!v->a[c].is_num()) return false;
        out[c] = v->a[c].num();
    }
    return true;
}

struct TomlParser {
    const std::string& s;
    size_t p = 0;
    int line = 1;
    std::string err;
    explicit TomlParser(const std::string& text) : s(text) {}

    bool fail(const std::string& m) {
        if (err.empty()) err = "line " + std::to_string(line) + ": " + m;
        return false;
    }
    bool eof() const { return p >= s.size(); }
    char c() const { return p < s.size() ? s[p] : '\0'; }
    void skip_ws() { while (!eof() && (c() == ' ' || c() == '\t' || c() == '\r')) ++p; }
    void skip_comment() { if (c() == '#') while (!eof() && c() != '\n') ++p; }
    void skip_ws_nl() {  // inside arrays: whitespace, newlines and comments
        for (;;) {
            skip_ws();
            skip_comment();
            if (c() == '\n') { ++p; ++line; continue; }
            break;
        }
    }
    bool end_of_line() {
        skip_ws();
        skip_comment();
        if (eof()) return true;
        if (c() == '\n') { ++p; ++line; return true; }
        return fail("unexpected text after a value");
    }

    bool key_part(std::string& k) {
        skip_ws();
        if (c() == '"' || c() == '\'') {
            TVal v;
            if (!string(v)) return false;
            k = v.s;
        } else {
            size_t b = p;
            while (!eof() && (isalnum((unsigned char)c()) || c() == '_' || c() == '-')) ++p;
            if (p == b) return fail("expected a key");
            k = s.substr(b, p - b);
        }
        skip_ws();
        return true;
    }
    bool key(std::vector<std::string>& ks) {
        ks.clear();
        for (;;) {
            std::string k;
            if (!key_part(k)) return false;
            ks.push_back(k);
            if (c() != '.') return true;
            ++p;
        }
    }

    bool string(TVal& v) {
        v.k = TVal::Str;
        char q = c();
        bool multi = s.compare(p, 3, std::string(3, q)) == 0;
        if (multi) {
            p += 3;
            if (c() == '\r') ++p;
            if (c() == '\n') { ++p; ++line; }
            std::string end(3, q);
            size_t e = s.find(end, p);
            if (e == std::string::npos) return fail("unterminated multi-line string");
            while (e + 3 < s.size() && s[e + 3] == q) ++e;  // up to two quotes may end the content
            std::string body = s.substr(p, e - p);
            for (char ch : body) if (ch == '\n') ++line;
            p = e + 3;
            if (q == '\'') { v.s = body; return true; }
            return unescape(body, v.s);
        }
        ++p;
        size_t b = p;
        if (q == '\'') {
            while (!eof() && c() != '\'' && c() != '\n') ++p;
            if (c() != '\'') return fail("unterminated string");
            v.s = s.substr(b, p - b);
            ++p;
            return true;
        }
        while (!eof() && c() != '"' && c() != '\n') p += (c() == '\\') ? 2 : 1;
        if (c() != '"') return fail("unterminated string");
        std::string body = s.substr(b, p - b);
        ++p;
        return unescape(body, v.s);
    }
    bool unescape(const std::string& in, std::string& out) {
        out.clear();
        for (size_t i = 0; i < in.size(); ++i) {
            if (in[i] != '\\') { out += in[i]; continue; }
            if (++i >= in.size()) return fail("bad escape");
            char e = in[i];
            switch (e) {
                case 'n': out += '\n'; break;
                case 't': out += '\t'; break;
                case 'r': out += '\r'; break;
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case '\n': while (i + 1 < in.size() && isspace((unsigned char)in[i + 1])) ++i; break;
                case 'u': case 'U': {
                    size_t nd = e == 'u' ? 4 : 8;
                    if (i + nd > in.size() - 1) return fail("bad unicode escape");
                    uint32_t cp = 0;
                    for (size_t k = 1; k <= nd; ++k) {
                        char h = in[i + k];
                        int dv = isdigit((unsigned char)h) ? h - '0'
                                 : (h >= 'a' && h <= 'f') ? h - 'a' + 10
                                 : (h >= 'A' && h <= 'F') ? h - 'A' + 10 : -1;
                        if (dv < 0) return fail("bad unicode escape");
                        cp = cp * 16 + (uint32_t)dv;
                    }
                    i += nd;
                    if (cp < 0x80) out += (char)cp;
                    else if (cp < 0x800) { out += (char)(0xc0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3f)); }
                    else if (cp < 0x10000) {
                        out += (char)(0xe0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3f));
                        out += (char)(0x80 | (cp & 0x3f));
                    } else {
                        out += (char)(0xf0 | (cp >> 18)); out += (char)(0x80 | ((cp >> 12) & 0x3f));
                        out += (char)(0x80 | ((cp >> 6) & 0x3f)); out += (char)(0x80 | (cp & 0x3f));
                    }
                    break;
                }
                default: return fail("bad escape");
            }
        }
        return true;
    }

    bool number(TVal& v) {
        size_t b = p;
        while (!eof() && (isalnum((unsigned char)c()) || c() == '+' || c() == '-' || c() == '.' || c() == '_')) ++p;
        std::string t;
        for (size_t i = b; i < p; ++i)
            if (s[i] != '_') t += s[i];
        if (t == "true") { v.k = TVal::Bool; v.b = true; return true; }
        if (t == "false") { v.k = TVal::Bool; v.b = false; return true; }
        std::string u = t;
        if (!u.empty() && (u[0] == '+' || u[0] == '-')) u = u.substr(1);
        if (u == "inf" || u == "nan") {
            v.k = TVal::Float;
            v.f = u == "inf" ? INFINITY : NAN;
            if (t[0] == '-') v.f = -v.f;
            return true;
        }
        if (t.empty()) return fail("expected a value");
        bool is_float = t.find_first_of(".eE") != std::string::npos && t.rfind("0x", 0) != 0;
        char* end = nullptr;
        if (is_float) {
            v.k = TVal::Float;
            v.f = std::strtod(t.c_str(), &end);
        } else {
            v.k = TVal::Int;
            int base = 10;
            std::string digits = t;
            bool neg = false;
            if (!digits.empty() && (digits[0] == '+' || digits[0] == '-')) { neg = digits[0] == '-'; digits = digits.substr(1); }
            if (digits.rfind("0x", 0) == 0) { base = 16; digits = digits.substr(2); }
            else if (digits.rfind("0o", 0) == 0) { base = 8; digits = digits.substr(2); }
            else if (digits.rfind("0b", 0) == 0) { base = 2; digits = digits.substr(2); }
            v.i = (int64_t)std::strtoll(digits.c_str(), &end, base);
            if (neg) v.i = -v.i;
        }
        if (!end || *end != '\0') return fail("bad number '" + t + "'");
        return true;
    }

    bool value(TVal& v) {
        skip_ws();
        char ch = c();
        if (ch == '"' || ch == '\'') return string(v);
        if (ch == '[') {
            ++p;
            v.k = TVal::Arr;
            for (;;) {
                skip_ws_nl();
                if (c() == ']') { ++p; return true; }
                TVal e;
                if (!value(e)) return false;
                v.a.push_back(std::move(e));
                skip_ws_nl();
                if (c() == ',') { ++p; continue; }
                if (c() == ']') { ++p; return true; }
                return fail("expected ',' or ']' in an array");
            }
        }
        if (ch == '{') {
            ++p;
            v.k = TVal::Tab;
            skip_ws();
            if (c() == '}') { ++p; return true; }
            for (;;) {
                std::vector<std::string> ks;
                if (!key(ks)) return false;
                if (c() != '=') return fail("expected '=' in an inline table");
                ++p;
                TVal* dst = &v;
                for (size_t i = 0; i + 1 < ks.size(); ++i) {
                    dst = dst->slot(ks[i]);
                    if (dst->k == TVal::None) dst->k = TVal::Tab;
                }
                TVal* leaf = dst->slot(ks.back());
                if (!value(*leaf)) return false;
                skip_ws();
                if (c() == ',') { ++p; continue; }
                if (c() == '}') { ++p; return true; }
                return fail("expected ',' or '}' in an inline table");
            }
        }
        return number(v);
    }

    // Walks dotted table keys from the root; arrays of tables resolve to their last element.
    TVal* walk(TVal& root, const std::vector<std::string>& ks, size_t upto) {
        TVal* cur = &root;
        for (size_t i = 0; i < upto; ++i) {
            TVal* nx = cur->slot(ks[i]);
            if (nx->k == TVal::None) nx->k = TVal::Tab;
            if (nx->k == TVal::Arr) {
                if (nx->a.empty() || nx->a.back().k != TVal::Tab) { fail("key is not a table"); return nullptr; }
                nx = &nx->a.back();
            }
            if (nx->k != TVal::Tab) { fail("key '" + ks[i] + "' is not a table"); return nullptr; }
            cur = nx;
        }
        return cur;
    }

    bool parse(TVal& root) {
        root = TVal{};
        root.k = TVal::Tab;
        TVal* cur = &root;
        while (!eof()) {
            skip_ws();
            skip_comment();
            if (eof()) break;
            if (c() == '\n') { ++p; ++line; continue; }
            if (c() == '[') {
                bool arr = s.compare(p, 2, "[[") == 0;
                p += arr ? 2 : 1;
                std::vector<std::string> ks;
                if (!key(ks)) return false;
                if (arr ? s.compare(p, 2, "]]") != 0 : c() != ']') return fail("unterminated table header");
                p += arr ? 2 : 1;
                TVal* parent = walk(root, ks, ks.size() - 1);
                if (!parent) return false;
                TVal* t = parent->slot(ks.back());
                if (arr) {
                    if (t->k == TVal::None) t->k = TVal::Arr;
                    if (t->k != TVal::Arr) return fail("'" + ks.back() + "' is not an array of tables");
                    t->a.emplace_back();
                    t->a.back().k = TVal::Tab;
                    cur = &t->a.back();
                } else {
                    if (t->k == TVal::None) t->k = TVal::Tab;
                    if (t->k == TVal::Arr && !t->a.empty()) t = &t->a.back();
                    if (t->k != TVal::Tab) return fail("'" + ks.back() + "' is not a table");
                    cur = t;
                }
                if (!end_of_line()) return false;
                continue;
            }
            std::vector<std::string> ks;
            if (!key(ks)) return false;
            if (c() != '=') return fail("expected '='");
            ++p;
            TVal* dst = cur;
            for (size_t i = 0; i + 1 < ks.size(); ++i) {
                dst = dst->slot(ks[i]);
                if (dst->k == TVal::None) dst->k = TVal::Tab;
                if (dst->k != TVal::Tab) return fail("dotted key through a non-table");
            }
            TVal* leaf = dst->slot(ks.back());
            if (leaf->k != TVal::None) return fail("duplicate key '" + ks.back() + "'");
            if (!value(*leaf)) return false;
            if (!end_of_line()) return false;
        }
        return true;
    }
};

bool parse_toml_text(const std::string& text, TVal& root, std::string& err) {
    TomlParser tp(text);
    if (!tp.parse(root)) { err = tp.err; return false; }
    return true;
}

bool read_file(const std::string& path, std::string& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

// ============================================================ project ====
// 3x4 affine transform, column vectors: p' = L p + T.
struct Affine {
    double L[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double T[3] = {0, 0, 0};
    Affine operator*(const Affine& o) const {
        Affine r;
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) r.L[i][j] = L[i][0] * o.L[0][j] + L[i][1] * o.L[1][j] + L[i][2] * o.L[2][j];
            r.T[i] = L[i][0] * o.T[0] + L[i][1] * o.T[1] + L[i][2] * o.T[2] + T[i];
        }
        return r;
    }
    void apply(const double* p, double* o) const {
        for (int i = 0; i < 3; ++i) o[i] = L[i][0] * p[0] + L[i][1] * p[1] + L[i][2] * p[2] + T[i];
    }
    void linear(const double* d, double* o) const {
        for (int i = 0; i < 3; ++i) o[i] = L[i][0] * d[0] + L[i][1] * d[1] + L[i][2] * d[2];
    }
    // normals: the inverse transpose of L (cofactors over the determinant), as the reference's hit shader
    // takes an object normal to the world with WorldToObject4x3 (raytracing/hit.hlsl:158); false when L is
    // singular
    bool normal(const double* n, double* o) const {
        double C[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
                C[i][j] = L[i1][j1] * L[i2][j2] - L[i1][j2] * L[i2][j1];
            }
        double det = L[0][0] * C[0][0] + L[0][1] * C[0][1] + L[0][2] * C[0][2];
        if (!(std::fabs(det) > 0.0)) return false;
        for (int i = 0; i < 3; ++i) o[i] = (C[i][0] * n[0] + C[i][1] * n[1] + C[i][2] * n[2]) / det;
        return true;
    }
    // rotation part (columns of L normalised): Transform::from_matrix, transform.cpp:36-47
    void rotate(const double* d, double* o) const {
        double cl[3];
        for (int j = 0; j < 3; ++j) {
            cl[j] = std::sqrt(L[0][j] * L[0][j] + L[1][j] * L[1][j] + L[2][j] * L[2][j]);
            if (cl[j] == 0.0) cl[j] = 1.0;
        }
        for (int i = 0; i < 3; ++i) o[i] = L[i][0] / cl[0] * d[0] + L[i][1] / cl[1] * d[1] + L[i][2] / cl[2] * d[2];
    }
};

// Transform component (math/transform.cpp:120-124): rotation = eulerAngleZXY(z, x, y)
// of the degree angles = Rz(z) Rx(x) Ry(y); matrix = [R * diag(scaling) | translation].
Affine transform_from(const TVal* v) {
    Affine a;
    if (!v) return a;
    double t[3] = {0, 0, 0}, r[3] = {0, 0, 0}, s[3] = {1, 1, 1};
    vec_of(v->get("translation"), 3, t);
    vec_of(v->get("rotation"), 3, r);
    vec_of(v->get("scaling"), 3, s);
    const double d2r = 3.14159265358979323846 / 180.0;
    double cx = std::cos(r[0] * d2r), sx = std::sin(r[0] * d2r);
    double cy = std::cos(r[1] * d2r), sy = std::sin(r[1] * d2r);
    double cz = std::cos(r[2] * d2r), sz = std::sin(r[2] * d2r);
    double Rz[3][3] = {{cz, -sz, 0}, {sz, cz, 0}, {0, 0, 1}};
    double Rx[3][3] = {{1, 0, 0}, {0, cx, -sx}, {0, sx, cx}};
    double Ry[3][3] = {{cy, 0, sy}, {0, 1, 0}, {-sy, 0, cy}};
    double ZX[3][3], R[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) ZX[i][j] = Rz[i][0] * Rx[0][j] + Rz[i][1] * Rx[1][j] + Rz[i][2] * Rx[2][j];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R[i][j] = ZX[i][0] * Ry[0][j] + ZX[i][1] * Ry[1][j] + ZX[i][2] * Ry[2][j];
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) a.L[i][j] = R[i][j] * s[j];
        a.T[i] = t[i];
    }
    return a;
}

struct ProjectOwned {
    std::vector<float> pos;
    std::vector<float> nrm;      // world-space vertex normals (zero for meshes without normals)
    bool any_normals = false;
    std::vector<uint32_t> idx, mat;
    std::vector<bsm_material> mats;
    std::vector<bsm_dir_light> lights;
    std::vector<bsm_point_light> points;
    std::vector<bsm_rect_light> rects;
};
std::mutex g_proj_mu;
std::unordered_map<const void*, ProjectOwned*> g_proj;  // keyed by desc->positions
std::mutex g_mesh_mu;
std::unordered_map<const void*, MeshOwned*> g_mesh;     // keyed by mesh->handle

// "/project/x/y" -> "<dir>/x/y"; other absolute paths are kept, relative ones joined.
std::string resolve(const std::string& dir, const std::string& path) {
    const std::string pre = "/project/";
    if (path.rfind(pre, 0) == 0) return dir + "/" + path.substr(pre.size());
    if (!path.empty() && path[0] == '/') return path;
    return dir + "/" + path;
}

bool load_toml(const std::string& path, TVal& root, std::string& err) {
    std::string text;
    if (!read_file(path, text)) { err = "cannot read " + path; return false; }
    if (!parse_toml_text(text, root, err)) { err = path + ": " + err; return false; }
    return true;
}

// Material TOML (material.cpp:12-53) to the pass's constant material.  The
// material function is HLSL; assignments of a parameter or a literal to
// surface.base_color / roughness / f0_color / opacity are evaluated, the blend
// mode selects the any-hit rule, and a `metallic`
// parameter with no f0 assignment gives f0 = lerp(0.04, base, metallic)
// (import_model.cpp:217-219).  Anything else (texture samples, expressions,
// conditionals) leaves the surface_data_default value of that field
// (material/utils.hlsl:18-31) and counts the material as approximated.
struct MatResult {
    bsm_material m;
    bool approximated = false;
    bool non_opaque = false;
};

std::string trim(const std::string& x, const char* ws = " \t\r\n") {
    size_t b = x.find_first_not_of(ws);
    if (b == std::string::npos) return "";
    size_t e = x.find_last_not_of(ws);
    return x.substr(b, e - b + 1);
}

bool param_value(const std::map<std::string, std::vector<double>>& params, const std::string& expr,
                 std::vector<double>& out) {
    std::string e = trim(expr);
    if (e.rfind("PARAM_", 0) == 0) {
        auto it = params.find(e.substr(6));
        if (it == params.end()) return false;
        out = it->second;
        return true;
    }
    // float3(a, b, c) / float(a) / a literal number
    size_t lp = e.find('(');
    std::string body = e;
    if (lp != std::string::npos) {
        std::string fn = e.substr(0, lp);
        if ((fn != "float3" && fn != "float" && fn != "float4") || e.back() != ')') return false;
        body = e.substr(lp + 1, e.size() - lp - 2);
    }
    out.clear();
    std::stringstream ss(body);
    std::string tok;
    while (std::getline(ss, tok, ',')) {
        char* end = nullptr;
        tok = trim(tok);
        if (!tok.empty() && (tok.back() == 'f' || tok.back() == 'F')) tok.pop_back();  // 1.0f
        double v = std::strtod(tok.c_str(), &end);
        if (tok.empty() || !end || *end != '\0') return false;
        out.push_back(v);
    }
    return !out.empty();
}

bool load_material(const std::string& path, MatResult& r, std::string& err) {
    TVal root;
    if (!load_toml(path, root, err)) return false;
    std::map<std::string, std::vector<double>> params;
    if (const TVal* ps = root.get("params"); ps && ps->k == TVal::Arr) {
        for (const TVal& pv : ps->a) {
            const TVal* nm = pv.get("name");
            const TVal* vv = pv.get("value");
            if (!nm || nm->k != TVal::Str || !vv) continue;
            if (vv->is_num()) params[nm->s] = {vv->num()};
            else if (vv->k == TVal::Arr) {
                std::vector<double> v;
                for (const TVal& e : vv->a)
                    if (e.is_num()) v.push_back(e.num());
                if (v.size() == vv->a.size()) params[nm->s] = v;
            } else if (vv->k == TVal::Tab) {
                r.approximated = true;  // texture parameter
            }
        }
    }
    const TVal* bm = root.get("blend_mode");
    uint32_t blend = BSM_BLEND_OPAQUE;
    if (bm && bm->k == TVal::Str) {
        if (bm->s == "alpha_test") blend = BSM_BLEND_ALPHA_TEST;
        else if (bm->s == "translucent") blend = BSM_BLEND_TRANSLUCENT;
        else if (bm->s != "opaque") { err = path + ": unknown blend_mode '" + bm->s + "'"; return false; }
    }
    r.non_opaque = blend != BSM_BLEND_OPAQUE;
    double base[3] = {0.5, 0.5, 0.5}, rough = 0.5, f0[3] = {0.04, 0.04, 0.04}, opacity = 1.0;
    bool has_f0 = false;
    const TVal* fn = root.get("material_function");
    std::string code = fn && fn->k == TVal::Str ? fn->s : "";
    std::stringstream ss(code);
    std::string stmt;
    while (std::getline(ss, stmt, ';')) {
        std::string st = trim(stmt);
        if (st.empty()) continue;
        size_t eq = st.find('=');
        std::string lhs = eq == std::string::npos ? "" : trim(st.substr(0, eq));
        std::vector<double> v;
        bool ok = eq != std::string::npos && st[eq + 1] != '=' && param_value(params, st.substr(eq + 1), v);
        if (ok && lhs == "surface.base_color" && v.size() >= 3) { for (int c = 0; c < 3; ++c) base[c] = v[c]; continue; }
        if (ok && lhs == "surface.roughness" && v.size() == 1) { rough = v[0]; continue; }
        if (ok && lhs == "surface.f0_color" && v.size() >= 3) { for (int c = 0; c < 3; ++c) f0[c] = v[c]; has_f0 = true; continue; }
        if (ok && lhs == "surface.opacity" && v.size() == 1) { opacity = v[0]; continue; }
        if (lhs == "surface.two_sided") continue;  // the pass faces every normal towards the ray
        r.approximated = true;
    }
    double metallic = 0.0;
    if (!has_f0) {
        auto it = params.find("metallic");
        if (it != params.end() && it->second.size() == 1) metallic = it->second[0];
    } else {
        // express the assigned f0 through the descriptor's metallic: exact when f0 is grey 0.04
        // or equals the base colour; otherwise the nearest metallic (least squares)
        double num = 0.0, den = 0.0;
        for (int c = 0; c < 3; ++c) { num += (f0[c] - 0.04) * (base[c] - 0.04); den += (base[c] - 0.04) * (base[c] - 0.04); }
        metallic = den > 0.0 ? std::min(1.0, std::max(0.0, num / den)) : 0.0;
        for (int c = 0; c < 3; ++c)
            if (std::fabs(0.04 + (base[c] - 0.04) * metallic - f0[c]) > 1e-6) r.approximated = true;
    }
    for (int c = 0; c < 3; ++c) { r.m.base_color[c] = (float)base[c]; r.m.emission[c] = 0.0f; }
    r.m.roughness = (float)rough;
    r.m.metallic = (float)metallic;
    r.m.opacity = (float)std::min(1.0, std::max(0.0, opacity));
    r.m.blend_mode = blend;
    return true;
}

}  // namespace

// ============================================================== C ABI ====
extern "C" bsm_status bsm_static_mesh_read(const void* bytes, uint64_t size, bsm_mesh_data* mesh, char* error,
                                           uint32_t error_len) {
    auto set_err = [&](const std::string& m) {
        if (error && error_len) { std::snprintf(error, error_len, "%s", m.c_str()); }
    };
    if (!bytes || !mesh) { set_err("null argument"); return BSM_ERR_INVALID_ARG; }
    std::unique_ptr<MeshOwned> m(new MeshOwned());
    std::string err;
    bool ok = false;
    try {
        ok = read_static_mesh((const uint8_t*)bytes, (size_t)size, *m, err);
    } catch (const std::exception& e) {
        err = e.what();
    }
    if (!ok) {
        set_err(err);
        return BSM_ERR_INVALID_ARG;
    }
    std::memset(mesh, 0, sizeof(*mesh));
    mesh->num_vertices = (uint32_t)(m->pos.size() / 3);
    mesh->positions = m->pos.data();
    mesh->normals = m->nrm.empty() ? nullptr : m->nrm.data();
    mesh->tangents = m->tan.empty() ? nullptr : m->tan.data();
    mesh->colors = m->col.empty() ? nullptr : m->col.data();
    mesh->num_normals = (uint32_t)(m->nrm.size() / 3);
    mesh->num_tangents = (uint32_t)(m->tan.size() / 4);
    mesh->num_colors = (uint32_t)(m->col.size() / 3);
    mesh->num_texcoords = (uint32_t)(m->uv.size() / 2);
    mesh->num_texcoords2 = (uint32_t)(m->uv2.size() / 2);
    mesh->texcoords = m->uv.empty() ? nullptr : m->uv.data();
    mesh->texcoords2 = m->uv2.empty() ? nullptr : m->uv2.data();
    mesh->num_indices = (uint32_t)m->idx.size();
    mesh->indices = m->idx.empty() ? nullptr : m->idx.data();
    mesh->num_submeshes = (uint32_t)m->sub.size();
    mesh->submeshes = m->sub.empty() ? nullptr : m->sub.data();
    std::lock_guard<std::mutex> lk(g_mesh_mu);
    mesh->handle = (void*)m.get();
    g_mesh[mesh->handle] = m.release();
    return BSM_OK;
}

extern "C" void bsm_static_mesh_free(bsm_mesh_data* mesh) {
    if (!mesh || !mesh->handle) return;
    MeshOwned* m = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mesh_mu);
        auto it = g_mesh.find(mesh->handle);
        if (it == g_mesh.end()) return;
        m = it->second;
        g_mesh.erase(it);
    }
    delete m;
    std::memset(mesh, 0, sizeof(*mesh));
}

extern "C" bsm_status bsm_static_mesh_write(const bsm_mesh_data* mesh, uint32_t version, void* out, uint64_t out_capacity,
                                            uint64_t* out_size) {
    if (!mesh || !out_size || (version != 1 && version != 2)) return BSM_ERR_INVALID_ARG;
    Writer body;
    body.arr(mesh->positions, mesh->positions ? mesh->num_vertices : 0, 12);
    body.arr(mesh->normals, mesh->normals ? mesh->num_normals : 0, 12);
    body.arr(mesh->tangents, mesh->tangents ? mesh->num_tangents : 0, 16);
    body.arr(mesh->colors, mesh->colors ? mesh->num_colors : 0, 12);
    body.arr(mesh->texcoords, mesh->texcoords ? mesh->num_texcoords : 0, 8);
    body.arr(mesh->texcoords2, mesh->texcoords2 ? mesh->num_texcoords2 : 0, 8);
    body.arr(mesh->indices, mesh->indices ? mesh->num_indices : 0, 4);
    std::vector<SubmeshRaw> sub(mesh->submeshes ? mesh->num_submeshes : 0);
    for (size_t i = 0; i < sub.size(); ++i) {
        const bsm_submesh& s = mesh->submeshes[i];
        sub[i] = SubmeshRaw{s.base_vertex, s.index_offset, s.num_indices, (uint8_t)s.topology, {0, 0, 0}};
    }
    body.arr(sub.data(), sub.size(), sizeof(SubmeshRaw));
    Writer w;
    w.put<uint32_t>(kAssetMagic);
    w.str(kMeshType);
    w.put<uint32_t>(version);
    if (version == 1) {
        w.raw(body.b.data(), body.b.size());
    } else {
        std::vector<uint8_t> z = zlib_store(body.b.data(), body.b.size());
        w.put<uint64_t>(body.b.size());
        w.put<uint64_t>(z.size());
        w.raw(z.data(), z.size());
    }
    *out_size = w.b.size();
    if (!out) return BSM_OK;
    if (out_capacity < w.b.size()) return BSM_ERR_INVALID_ARG;
    std::memcpy(out, w.b.data(), w.b.size());
    return BSM_OK;
}

namespace {
bsm_status project_load(const char* project_dir, bsm_scene_desc* desc, bsm_project_info* info);
}

extern "C" bsm_status bsm_project_load(const char* project_dir, bsm_scene_desc* desc, bsm_project_info* info) {
    if (!project_dir || !desc || !info) return BSM_ERR_INVALID_ARG;
    try {
        return project_load(project_dir, desc, info);
    } catch (const std::exception& e) {
        std::snprintf(info->error, sizeof(info->error), "%s", e.what());
        return BSM_ERR_INVALID_ARG;
    }
}

namespace {
bsm_status project_load(const char* project_dir, bsm_scene_desc* desc, bsm_project_info* info) {
    std::memset(info, 0, sizeof(*info));
    bsm_pt_settings_default(&info->settings);
    info->near_z = 0.01f;
    info->far_z = 10000.0f;
    auto fail = [&](const std::string& m) {
        std::snprintf(info->error, sizeof(info->error), "%s", m.c_str());
        return BSM_ERR_INVALID_ARG;
    };
    std::string dir = project_dir;
    while (dir.size() > 1 && dir.back() == '/') dir.pop_back();
    std::string err;
    TVal project;
    if (!load_toml(dir + "/project.toml", project, err)) return fail(err);
    const TVal* sf = project.get("scene_file");
    const TVal* mf = project.get("asset_metadata_file");
    if (!sf || sf->k != TVal::Str || !mf || mf->k != TVal::Str)
        return fail("project.toml lacks scene_file / asset_metadata_file");
    TVal meta, scene;
    if (!load_toml(resolve(dir, mf->s), meta, err)) return fail(err);
    if (!load_toml(resolve(dir, sf->s), scene, err)) return fail(err);
    std::map<int64_t, std::pair<std::string, std::string>> assets;  // id -> (path, type)
    if (const TVal* as = meta.get("assets"); as && as->k == TVal::Arr)
        for (const TVal& a : as->a) {
            const TVal* id = a.get("id");
            const TVal* pth = a.get("path");
            const TVal* ty = a.get("type");
            if (id && id->k == TVal::Int && pth && pth->k == TVal::Str)
                assets[id->i] = {resolve(dir, pth->s), ty && ty->k == TVal::Str ? ty->s : ""};
        }
    auto asset_path = [&](const TVal* ref, const char* type, std::string& out) {
        const TVal* id = ref ? ref->get("asset_id") : nullptr;
        if (!id || id->k != TVal::Int) return false;
        auto it = assets.find(id->i);
        if (it == assets.end() || (type && it->second.second != type)) return false;
        out = it->second.first;
        return true;
    };

    const TVal* objs = scene.get("objects");
    size_t nobj = objs && objs->k == TVal::Arr ? objs->a.size() : 0;
    info->num_objects = (uint32_t)nobj;
    // world transforms: parent index into the objects array (scene.cpp:111-134)
    std::vector<Affine> local(nobj), world(nobj);
    std::vector<int> parent(nobj, -1);
    for (size_t i = 0; i < nobj; ++i) {
        const TVal& o = objs->a[i];
        if (const TVal* pv = o.get("parent"); pv && pv->k == TVal::Int) parent[i] = (int)pv->i;
        if (const TVal* cs = o.get("components"); cs && cs->k == TVal::Arr)
            for (const TVal& c : cs->a) {
                const TVal* ty = c.get("type");
                if (ty && ty->k == TVal::Str && ty->s == "Transform") local[i] = transform_from(c.get("value"));
            }
    }
    std::vector<int> state(nobj, 0);  // 0 todo, 1 in progress, 2 done
    std::function<bool(size_t)> resolve_world = [&](size_t i) -> bool {
        if (state[i] == 2) return true;
        if (state[i] == 1) return false;  // cycle
        state[i] = 1;
        int pa = parent[i];
        if (pa >= 0 && (size_t)pa < nobj) {
            if (!resolve_world((size_t)pa)) return false;
            world[i] = world[(size_t)pa] * local[i];
        } else {
            world[i] = local[i];
        }
        state[i] = 2;
        return true;
    };
    for (size_t i = 0; i < nobj; ++i)
        if (!resolve_world(i)) return fail("cycle in the objects' parent links");

    std::unique_ptr<ProjectOwned> own(new ProjectOwned());
    std::map<std::string, uint32_t> mat_index;
    std::map<std::string, std::shared_ptr<MeshOwned>> mesh_cache;
    for (size_t i = 0; i < nobj; ++i) {
        const TVal* cs = objs->a[i].get("components");
        if (!cs || cs->k != TVal::Arr) continue;
        const TVal *mesh_c = nullptr, *rend_c = nullptr;
        for (const TVal& c : cs->a) {
            const TVal* ty = c.get("type");
            const TVal* val = c.get("value");
            if (!ty || ty->k != TVal::Str || !val) continue;
            const std::string& t = ty->s;
            if (t == "CameraComponent" && !info->has_camera) {
                // camera_system.cpp:17-29: position, front = -z, up = +y of the world transform
                double o0[3] = {0, 0, 0}, pz[3], fz[3] = {0, 0, -1}, uy[3] = {0, 1, 0}, f[3], u[3];
                world[i].apply(o0, pz);
                world[i].linear(fz, f);
                world[i].linear(uy, u);
                bsm_camera& cam = info->camera;
                for (int k = 0; k < 3; ++k) {
                    cam.position[k] = (float)pz[k];
                    cam.front[k] = (float)f[k];
                    cam.up[k] = (float)u[k];
                }
                cam.yfov_deg = (float)num_or(val->get("yfov"), 30.0);
                double size[2] = {0, 0};
                vec_of(val->get("render_target_size"), 2, size);
                cam.width = (uint32_t)size[0];
                cam.height = (uint32_t)size[1];
                info->near_z = (float)num_or(val->get("near_z"), 0.01);
                info->far_z = (float)num_or(val->get("far_z"), 10000.0);
                const TVal* pt = val->get("projection_type");
                info->camera_orthographic = pt && pt->k == TVal::Str && pt->s == "orthographic";
                info->has_camera = 1;
            } else if (t == "DirectionalLightComponent") {
                // lights.cpp:55-65: emission = colour * strength (skipped when zero),
                // direction = rotation * (0, 1, 0)
                double col[3] = {1, 1, 1};
                vec_of(val->get("color"), 3, col);
                double strength = num_or(val->get("strength"), 1.0);
                bsm_dir_light l;
                bool zero = true;
                for (int k = 0; k < 3; ++k) {
                    l.emission[k] = (float)(col[k] * strength);
                    zero = zero && l.emission[k] == 0.0f;
                }
                if (zero) continue;
                double y[3] = {0, 1, 0}, d[3];
                world[i].rotate(y, d);
                double n = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                for (int k = 0; k < 3; ++k) l.direction[k] = (float)(d[k] / n);
                own->lights.push_back(l);
            } else if (t == "StaticMeshComponent") {
                mesh_c = val;
            } else if (t == "MeshRendererComponent") {
                rend_c = val;
            } else if (t == "SkyboxComponent") {
                info->has_skybox = 1;
            } else if (t == "PointLightComponent") {
                // lights.cpp:120-139: position = translation, direction = rotation * (0, 1, 0),
                // spot cone cosines, 1 / range^2 attenuation
                double col[3] = {1, 1, 1};
                vec_of(val->get("color"), 3, col);
                double strength = num_or(val->get("strength"), 1.0);
                bsm_point_light pl{};
                bool zero = true;
                for (int k = 0; k < 3; ++k) {
                    pl.emission[k] = (float)(col[k] * strength);
                    zero = zero && pl.emission[k] == 0.0f;
                }
                if (zero) continue;
                double o0[3] = {0, 0, 0}, pw[3], y[3] = {0, 1, 0}, d[3];
                world[i].apply(o0, pw);
                world[i].rotate(y, d);
                double n = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                for (int k = 0; k < 3; ++k) { pl.position[k] = (float)pw[k]; pl.direction[k] = (float)(d[k] / n); }
                pl.range = (float)num_or(val->get("range"), 30.0);
                const TVal* spot = val->get("spot");
                if (spot && spot->k == TVal::Bool && spot->b) {
                    const double d2r = 3.14159265358979323846 / 180.0;
                    pl.cos_inner = (float)std::cos(num_or(val->get("spot_inner_angle"), 30.0) * d2r);
                    pl.cos_outer = (float)std::cos(num_or(val->get("spot_outer_angle"), 60.0) * d2r);
                }
                own->points.push_back(pl);
            } else if (t == "RectLightComponent") {
                // lights.cpp:210-228: centre = translation, corners along rotation * (+-w/2, +-h/2, 0)
                double col[3] = {1, 1, 1};
                vec_of(val->get("color"), 3, col);
                double strength = num_or(val->get("strength"), 1.0);
                bsm_rect_light rl{};
                bool zero = true;
                for (int k = 0; k < 3; ++k) {
                    rl.emission[k] = (float)(col[k] * strength);
                    zero = zero && rl.emission[k] == 0.0f;
                }
                if (zero) continue;
                double o0[3] = {0, 0, 0}, pw[3], x[3] = {1, 0, 0}, y[3] = {0, 1, 0}, ax[3], ay[3];
                world[i].apply(o0, pw);
                world[i].rotate(x, ax);
                world[i].rotate(y, ay);
                for (int k = 0; k < 3; ++k) {
                    rl.center[k] = (float)pw[k];
                    rl.axis_x[k] = (float)ax[k];
                    rl.axis_y[k] = (float)ay[k];
                }
                rl.width = (float)num_or(val->get("width"), 1.0);
                rl.height = (float)num_or(val->get("height"), 1.0);
                const TVal* ts = val->get("two_sided");
                rl.two_sided = ts && ts->k == TVal::Bool && ts->b ? 1u : 0u;
                if (const TVal* tex = val->get("texture"); tex && tex->k == TVal::Tab && tex->get("asset_id"))
                    info->num_unsupported_lights++;  // textured rect light: traced with its constant emission
                own->rects.push_back(rl);
            } else if (t == "BasicRendererOverrideVolume") {
                const TVal* st = val->get("settings");
                const TVal* pt = st ? st->get("path_tracing") : nullptr;
                if (pt) {
                    bsm_pt_settings& s = info->settings;
                    s.ray_length = (float)num_or(pt->get("ray_length"), s.ray_length);
                    s.max_bounces = (uint32_t)num_or(pt->get("max_bounces"), s.max_bounces);
                    if (const TVal* a = pt->get("accumulate"); a && a->k == TVal::Bool) s.accumulate = a->b;
                    if (const TVal* dn = pt->get("denoise"); dn && dn->k == TVal::Bool) s.denoise = dn->b;
                }
            }
        }
        if (!mesh_c || !rend_c) continue;
        std::string mpath;
        if (!asset_path(mesh_c->get("static_mesh"), "StaticMesh", mpath))
            return fail("object " + std::to_string(i) + ": static_mesh asset not in the metadata");
        std::shared_ptr<MeshOwned>& mo = mesh_cache[mpath];
        if (!mo) {
            std::string bytes;
            if (!read_file(mpath, bytes)) return fail("cannot read " + mpath);
            mo = std::make_shared<MeshOwned>();
            if (!read_static_mesh((const uint8_t*)bytes.data(), bytes.size(), *mo, err)) return fail(mpath + ": " + err);
        }
        // drawables: submesh start + i with material i (static_mesh_render_system.cpp:56-79)
        const TVal* mats = rend_c->get("materials");
        size_t nm = mats && mats->k == TVal::Arr ? mats->a.size() : 0;
        uint32_t start = (uint32_t)num_or(rend_c->get("submesh_start_index"), 0.0);
        size_t nsub = mo->sub.size() > start ? mo->sub.size() - start : 0;
        size_t ndraw = std::min(nm, nsub);
        const uint32_t nv = (uint32_t)(mo->pos.size() / 3);
        const uint32_t vbase = (uint32_t)(own->pos.size() / 3);
        bool placed = false;
        for (size_t d = 0; d < ndraw; ++d) {
            const bsm_submesh& sm = mo->sub[start + d];
            if (sm.topology != 3) { info->num_skipped_submeshes++; continue; }  // triangle_list only
            std::string matpath;
            if (!asset_path(&mats->a[d], "Material", matpath))
                return fail("object " + std::to_string(i) + ": material asset not in the metadata");
            uint32_t mid;
            auto mit = mat_index.find(matpath);
            if (mit == mat_index.end()) {
                MatResult mr;
                if (!load_material(matpath, mr, err)) return fail(err);
                mid = (uint32_t)own->mats.size();
                own->mats.push_back(mr.m);
                mat_index[matpath] = mid;
                info->num_materials_approximated += mr.approximated;
                info->num_non_opaque_materials += mr.non_opaque;
            } else {
                mid = mit->second;
            }
            if (!placed) {  // the object's vertices (and normals, where the mesh has them) in world space, once
                const bool has_n = mo->nrm.size() == 3 * (size_t)nv;
                for (uint32_t v = 0; v < nv; ++v) {
                    double p[3] = {mo->pos[3 * v], mo->pos[3 * v + 1], mo->pos[3 * v + 2]}, w[3];
                    world[i].apply(p, w);
                    for (int k = 0; k < 3; ++k) own->pos.push_back((float)w[k]);
                    double n[3] = {0, 0, 0}, wn[3] = {0, 0, 0};
                    if (has_n) {
                        n[0] = mo->nrm[3 * v]; n[1] = mo->nrm[3 * v + 1]; n[2] = mo->nrm[3 * v + 2];
                        if (!world[i].normal(n, wn)) wn[0] = wn[1] = wn[2] = 0.0;
                    }
                    for (int k = 0; k < 3; ++k) own->nrm.push_back((float)wn[k]);
                }
                own->any_normals = own->any_normals || has_n;
                placed = true;
            }
            // ~0 = to the end of the index data (mesh.cpp:84-87, graphics_manager.cpp:726-729)
            uint64_t count = sm.num_indices;
            if (sm.num_indices == ~0u)
                count = mo->idx.empty() ? (sm.base_vertex < nv ? nv - sm.base_vertex : 0)
                                        : (sm.index_offset < mo->idx.size() ? mo->idx.size() - sm.index_offset : 0);
            uint32_t ntri = (uint32_t)(count / 3);
            for (uint32_t t = 0; t < ntri; ++t)
                for (int k = 0; k < 3; ++k) {
                    uint64_t j = (uint64_t)sm.index_offset + 3ull * t + k;
                    uint64_t v;
                    if (mo->idx.empty()) {
                        v = (uint64_t)sm.base_vertex + 3ull * t + k;  // no index data: num_indices counts vertices
                    } else {
                        if (j >= mo->idx.size()) return fail(mpath + ": submesh indices out of range");
                        v = (uint64_t)sm.base_vertex + mo->idx[j];
                    }
                    if (v >= nv) return fail(mpath + ": vertex index out of range");
                    own->idx.push_back(vbase + (uint32_t)v);
                }
            for (uint32_t t = 0; t < ntri; ++t) own->mat.push_back(mid);
            info->num_drawables++;
        }
    }
    if (own->mats.empty()) {  // a scene without drawables still needs one material
        bsm_material m{{0.5f, 0.5f, 0.5f}, 0.5f, 0.0f, {0, 0, 0}, 1.0f, BSM_BLEND_OPAQUE};
        own->mats.push_back(m);
    }
    std::memset(desc, 0, sizeof(*desc));
    desc->num_vertices = (uint32_t)(own->pos.size() / 3);
    desc->positions = own->pos.empty() ? nullptr : own->pos.data();
    desc->num_triangles = (uint32_t)(own->idx.size() / 3);
    desc->indices = own->idx.empty() ? nullptr : own->idx.data();
    desc->material_ids = own->mat.empty() ? nullptr : own->mat.data();
    desc->num_materials = (uint32_t)own->mats.size();
    desc->materials = own->mats.data();
    desc->num_dir_lights = (uint32_t)own->lights.size();
    desc->dir_lights = own->lights.empty() ? nullptr : own->lights.data();
    desc->num_point_lights = (uint32_t)own->points.size();
    desc->point_lights = own->points.empty() ? nullptr : own->points.data();
    desc->num_rect_lights = (uint32_t)own->rects.size();
    desc->rect_lights = own->rects.empty() ? nullptr : own->rects.data();
    desc->normals = own->any_normals ? own->nrm.data() : nullptr;
    // no SkyboxComponent texture support: the reference's black 1x1 cube when none is set
    // (skybox.cpp:47-50)
    desc->sky.kind = BSM_SKY_CONSTANT;
    const void* key = desc->materials;
    std::lock_guard<std::mutex> lk(g_proj_mu);
    g_proj[key] = own.release();
    return BSM_OK;
}
}  // namespace

extern "C" void bsm_project_free(bsm_scene_desc* desc) {
    if (!desc || !desc->materials) return;
    ProjectOwned* own = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_proj_mu);
        auto it = g_proj.find(desc->materials);
        if (it == g_proj.end()) return;
        own = it->second;
        g_proj.erase(it);
    }
    delete own;
    std::memset(desc, 0, sizeof(*desc));
}

extern "C" bsm_status bsm_toml_check(const char* text, char* error, uint32_t error_len) {
    if (!text) return BSM_ERR_INVALID_ARG;
    TVal root;
    std::string err;
    bool ok = false;
    try {
        ok = parse_toml_text(text, root, err);
    } catch (const std::exception& e) {
        err = e.what();
    }
    if (!ok) {
        if (error && error_len) std::snprintf(error, error_len, "%s", err.c_str());
        return BSM_ERR_INVALID_ARG;
    }
    return BSM_OK;
}
