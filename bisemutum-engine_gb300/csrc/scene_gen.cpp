// scene_gen.cpp — seeded procedural scenes that stand in for the engine's
// asset-loaded scenes (the reference renders whatever the editor loads; these
// generators give the pass fixed, reproducible inputs of known size).
//
//  BSM_SCENE_ROOM:    an open Cornell-style room of 12 axis-aligned quads (floor,
//                     back, left and right walls, and the four sides of two
//                     blocks) plus N icospheres (subdivision 2, 320 triangles)
//                     with centres uniform in the room and radii uniform in
//                     [0.05, 0.2]; constant sky 0.5; one sun of irradiance 3.
//  BSM_SCENE_TERRAIN: a grid x grid fBm heightfield (6 octaves, heights in
//                     [0, 0.15]) plus N UV spheres (16 x 16 segments, 480
//                     triangles) placed on the terrain with radii in
//                     [0.005, 0.03]; a gradient sky baked into an RGBA16F
//                     equirect map; one sun of irradiance 3.
// Materials: albedo U[0.1, 0.9]^3, roughness U[0.05, 1], metallic Bernoulli(0.3).
#include "bsm_pt.h"

#include <algorithm>
#include <array>
#include <mutex>
#include <unordered_map>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

struct Rng {  // SplitMix64 stream
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
};

struct Builder {
    std::vector<float> pos;
    std::vector<uint32_t> idx;
    std::vector<uint32_t> mat;
    std::vector<bsm_material> mats;

    uint32_t vertex(double x, double y, double z) {
        pos.push_back((float)x); pos.push_back((float)y); pos.push_back((float)z);
        return (uint32_t)(pos.size() / 3 - 1);
    }
    void tri(uint32_t a, uint32_t b, uint32_t c, uint32_t m) {
        idx.push_back(a); idx.push_back(b); idx.push_back(c); mat.push_back(m);
    }
    uint32_t random_material(Rng& r) {
        bsm_material m{};
        for (int i = 0; i < 3; ++i) m.base_color[i] = (float)r.uniform(0.1, 0.9);
        m.roughness = (float)r.uniform(0.05, 1.0);
        m.metallic = r.uniform() < 0.3 ? 1.0f : 0.0f;
        m.opacity = 1.0f;
        m.blend_mode = BSM_BLEND_OPAQUE;
        mats.push_back(m);
        return (uint32_t)(mats.size() - 1);
    }
    // axis-aligned quad from corner o spanning edges a and b
    void quad(const double o[3], const double a[3], const double b[3], uint32_t m) {
        uint32_t v0 = vertex(o[0], o[1], o[2]);
        uint32_t v1 = vertex(o[0] + a[0], o[1] + a[1], o[2] + a[2]);
        uint32_t v2 = vertex(o[0] + a[0] + b[0], o[1] + a[1] + b[1], o[2] + a[2] + b[2]);
        uint32_t v3 = vertex(o[0] + b[0], o[1] + b[1], o[2] + b[2]);
        tri(v0, v1, v2, m);
        tri(v0, v2, v3, m);
    }
};

void normalize3(double v[3]) {
    double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= l; v[1] /= l; v[2] /= l;
}

// Icosphere: icosahedron subdivided `levels` times, 20 * 4^levels triangles.
void icosphere(Builder& b, const double c[3], double radius, int levels, uint32_t m) {
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<std::array<double, 3>> v = {
        {-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
        {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    std::vector<std::array<int, 3>> f = {
        {0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
        {11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8},
        {3, 8, 9}, {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    for (auto& p : v) { double q[3] = {p[0], p[1], p[2]}; normalize3(q); p = {q[0], q[1], q[2]}; }
    for (int l = 0; l < levels; ++l) {
        std::vector<std::array<int, 3>> nf;
        auto mid = [&](int a, int bb) {
            double q[3] = {(v[a][0] + v[bb][0]) * 0.5, (v[a][1] + v[bb][1]) * 0.5, (v[a][2] + v[bb][2]) * 0.5};
            normalize3(q);
            v.push_back({q[0], q[1], q[2]});
            return (int)v.size() - 1;
        };
        for (auto& tri : f) {
            int a = mid(tri[0], tri[1]), bb = mid(tri[1], tri[2]), cc = mid(tri[2], tri[0]);
            nf.push_back({tri[0], a, cc});
            nf.push_back({tri[1], bb, a});
            nf.push_back({tri[2], cc, bb});
            nf.push_back({a, bb, cc});
        }
        f.swap(nf);
    }
    uint32_t base = (uint32_t)(b.pos.size() / 3);
    for (auto& p : v) b.vertex(c[0] + radius * p[0], c[1] + radius * p[1], c[2] + radius * p[2]);
    for (auto& tri : f) b.tri(base + tri[0], base + tri[1], base + tri[2], m);
}

// UV sphere with `seg` slices and `seg` stacks: 2*seg + 2*seg*(seg-2) triangles
// (480 for seg = 16).
void uv_sphere(Builder& b, const double c[3], double radius, int seg, uint32_t m) {
    const double pi = 3.14159265358979323846;
    uint32_t top = b.vertex(c[0], c[1] + radius, c[2]);
    uint32_t ring0 = (uint32_t)(b.pos.size() / 3);
    for (int i = 1; i < seg; ++i) {
        double th = pi * i / seg;
        for (int j = 0; j < seg; ++j) {
            double ph = 2.0 * pi * j / seg;
            b.vertex(c[0] + radius * std::sin(th) * std::cos(ph), c[1] + radius * std::cos(th),
                     c[2] + radius * std::sin(th) * std::sin(ph));
        }
    }
    uint32_t bottom = b.vertex(c[0], c[1] - radius, c[2]);
    auto ring = [&](int i, int j) { return ring0 + (uint32_t)((i - 1) * seg + (j % seg)); };
    for (int j = 0; j < seg; ++j) b.tri(top, ring(1, j + 1), ring(1, j), m);
    for (int i = 1; i < seg - 1; ++i)
        for (int j = 0; j < seg; ++j) {
            b.tri(ring(i, j), ring(i, j + 1), ring(i + 1, j + 1), m);
            b.tri(ring(i, j), ring(i + 1, j + 1), ring(i + 1, j), m);
        }
    for (int j = 0; j < seg; ++j) b.tri(bottom, ring(seg - 1, j), ring(seg - 1, j + 1), m);
}

double lattice(int64_t x, int64_t y, uint64_t seed) {
    uint64_t h = seed ^ ((uint64_t)x * 0x9e3779b97f4a7c15ULL) ^ ((uint64_t)y * 0xc2b2ae3d27d4eb4fULL);
    h = (h ^ (h >> 30)) * 0xbf58476d1ce4e5b9ULL;
    h = (h ^ (h >> 27)) * 0x94d049bb133111ebULL;
    h ^= h >> 31;
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}
double value_noise(double x, double y, uint64_t seed) {
    double fx = std::floor(x), fy = std::floor(y);
    int64_t ix = (int64_t)fx, iy = (int64_t)fy;
    double tx = x - fx, ty = y - fy;
    tx = tx * tx * (3.0 - 2.0 * tx);
    ty = ty * ty * (3.0 - 2.0 * ty);
    double a = lattice(ix, iy, seed), b = lattice(ix + 1, iy, seed);
    double c = lattice(ix, iy + 1, seed), d = lattice(ix + 1, iy + 1, seed);
    return (a + (b - a) * tx) + ((c + (d - c) * tx) - (a + (b - a) * tx)) * ty;
}
double fbm(double x, double y, uint64_t seed) {
    double sum = 0.0, amp = 0.5, freq = 4.0;
    for (int o = 0; o < 6; ++o) {
        sum += amp * value_noise(x * freq, y * freq, seed + (uint64_t)o * 1315423911ULL);
        amp *= 0.5;
        freq *= 2.0;
    }
    return sum;
}

uint16_t float_to_half(float f) {  // round-to-nearest-even, finite positive range used here
    uint32_t x;
    std::memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    int32_t exp = (int32_t)((x >> 23) & 0xff) - 127 + 15;
    uint32_t man = x & 0x7fffffu;
    if (((x >> 23) & 0xff) == 0xff) return (uint16_t)(sign | 0x7c00u | (man ? 0x200u : 0u));
    if (exp >= 31) return (uint16_t)(sign | 0x7c00u);
    if (exp <= 0) {
        if (exp < -10) return (uint16_t)sign;
        man |= 0x800000u;
        uint32_t shift = (uint32_t)(14 - exp);
        uint32_t h = man >> shift;
        uint32_t rem = man & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (h & 1u))) ++h;
        return (uint16_t)(sign | h);
    }
    uint32_t h = ((uint32_t)exp << 10) | (man >> 13);
    uint32_t rem = man & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
}

void random_sun(Rng& r, bsm_dir_light& sun, float irradiance) {
    // uniform over the upper hemisphere (y > 0), kept a little above the horizon
    double z = r.uniform(0.15, 1.0);
    double phi = r.uniform(0.0, 2.0 * 3.14159265358979323846);
    double s = std::sqrt(1.0 - z * z);
    sun.direction[0] = (float)(s * std::cos(phi));
    sun.direction[1] = (float)z;
    sun.direction[2] = (float)(s * std::sin(phi));
    for (int i = 0; i < 3; ++i) sun.emission[i] = irradiance;
}

struct Owned {  // everything bsm_scene_desc points at, freed together
    std::vector<float> pos;
    std::vector<uint32_t> idx, mat;
    std::vector<bsm_material> mats;
    bsm_dir_light sun;
    std::vector<uint16_t> sky;
};

std::mutex g_owned_mu;
std::unordered_map<const void*, Owned*> g_owned;  // keyed by desc->positions

}  // namespace

extern "C" bsm_status bsm_scene_generate(const bsm_scene_gen_params* p, bsm_scene_desc* desc, bsm_camera* cam) {
    if (!p || !desc) return BSM_ERR_INVALID_ARG;
    Rng rng{p->seed * 0x2545f4914f6cdd1dULL + 0x1234567ULL};
    Builder b;
    Owned* own = new Owned();
    bsm_sky sky{};
    if (p->kind == BSM_SCENE_ROOM) {
        uint32_t n_spheres = p->spheres ? p->spheres : 64u;
        // room walls (open ceiling and open front at z = 0)
        const double O[3] = {0, 0, 0};
        const double X[3] = {1, 0, 0}, Y[3] = {0, 1, 0}, Z[3] = {0, 0, 1};
        { const double o[3] = {0, 0, 0}; b.quad(o, Z, X, b.random_material(rng)); }   // floor
        { const double o[3] = {0, 0, 1}; b.quad(o, X, Y, b.random_material(rng)); }   // back
        { b.quad(O, Y, Z, b.random_material(rng)); }                                   // left
        { const double o[3] = {1, 0, 0}; b.quad(o, Z, Y, b.random_material(rng)); }   // right
        // two blocks, four vertical sides each
        const double blocks[2][4] = {{0.15, 0.55, 0.3, 0.6}, {0.6, 0.35, 0.3, 0.3}};  // x, z, w(=d), h
        for (auto& bl : blocks) {
            uint32_t m = b.random_material(rng);
            double x0 = bl[0], z0 = bl[1], w = bl[2], h = bl[3];
            const double ex[3] = {w, 0, 0}, ez[3] = {0, 0, w}, ey[3] = {0, h, 0};
            const double nx[3] = {-w, 0, 0}, nz[3] = {0, 0, -w};
            { const double o[3] = {x0, 0, z0}; b.quad(o, ex, ey, m); }
            { const double o[3] = {x0 + w, 0, z0}; b.quad(o, ez, ey, m); }
            { const double o[3] = {x0 + w, 0, z0 + w}; b.quad(o, nx, ey, m); }
            { const double o[3] = {x0, 0, z0 + w}; b.quad(o, nz, ey, m); }
        }
        for (uint32_t i = 0; i < n_spheres; ++i) {
            double c[3] = {rng.uniform(), rng.uniform(), rng.uniform()};
            double r = rng.uniform(0.05, 0.2);
            icosphere(b, c, r, 2, b.random_material(rng));
        }
        random_sun(rng, own->sun, 3.0f);
        sky.kind = BSM_SKY_CONSTANT;
        sky.color[0] = sky.color[1] = sky.color[2] = 0.5f;
        if (cam) {
            const float pos[3] = {0.5f, 0.55f, -1.1f};
            const float tgt[3] = {0.5f, 0.4f, 0.5f};
            double f[3] = {tgt[0] - pos[0], tgt[1] - pos[1], tgt[2] - pos[2]};
            normalize3(f);
            for (int i = 0; i < 3; ++i) { cam->position[i] = pos[i]; cam->front[i] = (float)f[i]; }
            cam->up[0] = 0; cam->up[1] = 1; cam->up[2] = 0;
            cam->yfov_deg = 60.0f;
        }
    } else if (p->kind == BSM_SCENE_TERRAIN) {
        uint32_t G = p->grid ? p->grid : 512u;
        uint32_t n_spheres = p->spheres;
        if (G < 2) { delete own; return BSM_ERR_INVALID_ARG; }
        uint64_t nseed = rng.next();
        std::vector<double> h((size_t)G * G);
        double hmin = 1e30, hmax = -1e30;
        for (uint32_t j = 0; j < G; ++j)
            for (uint32_t i = 0; i < G; ++i) {
                double v = fbm((double)i / (G - 1), (double)j / (G - 1), nseed);
                h[(size_t)j * G + i] = v;
                hmin = std::min(hmin, v); hmax = std::max(hmax, v);
            }
        double scale = hmax > hmin ? 0.15 / (hmax - hmin) : 0.0;
        for (auto& v : h) v = (v - hmin) * scale;
        uint32_t terrain_mat = b.random_material(rng);
        for (uint32_t j = 0; j < G; ++j)
            for (uint32_t i = 0; i < G; ++i)
                b.vertex((double)i / (G - 1), h[(size_t)j * G + i], (double)j / (G - 1));
        for (uint32_t j = 0; j + 1 < G; ++j)
            for (uint32_t i = 0; i + 1 < G; ++i) {
                uint32_t a = j * G + i, bb = a + 1, c = a + G, d = c + 1;
                b.tri(a, c, d, terrain_mat);
                b.tri(a, d, bb, terrain_mat);
            }
        auto height_at = [&](double x, double z) {
            double fx = x * (G - 1), fz = z * (G - 1);
            uint32_t i = std::min((uint32_t)fx, G - 2), j = std::min((uint32_t)fz, G - 2);
            double tx = fx - i, tz = fz - j;
            double a = h[(size_t)j * G + i], bb = h[(size_t)j * G + i + 1];
            double c = h[(size_t)(j + 1) * G + i], d = h[(size_t)(j + 1) * G + i + 1];
            return (a + (bb - a) * tx) * (1 - tz) + (c + (d - c) * tx) * tz;
        };
        for (uint32_t s = 0; s < n_spheres; ++s) {
            double x = rng.uniform(0.02, 0.98), z = rng.uniform(0.02, 0.98);
            double r = rng.uniform(0.005, 0.03);
            double c[3] = {x, height_at(x, z) + 0.8 * r, z};
            uv_sphere(b, c, r, 16, b.random_material(rng));
        }
        random_sun(rng, own->sun, 3.0f);
        // gradient sky with a glow around the sun, baked to RGBA16F
        uint32_t W = p->sky_width ? p->sky_width : 1024u, H = p->sky_height ? p->sky_height : 512u;
        own->sky.resize((size_t)W * H * 4);
        const double pi = 3.14159265358979323846;
        const double zen[3] = {0.25, 0.45, 0.95}, hor[3] = {0.95, 0.95, 1.0}, gnd[3] = {0.35, 0.3, 0.25};
        for (uint32_t i = 0; i < H; ++i) {
            double th = pi * (i + 0.5) / H;
            for (uint32_t j = 0; j < W; ++j) {
                double ph = 2.0 * pi * ((j + 0.5) / W - 0.5);
                double d[3] = {std::sin(th) * std::cos(ph), std::cos(th), std::sin(th) * std::sin(ph)};
                double rgb[3];
                if (d[1] >= 0.0) {
                    double t = std::sqrt(d[1]);
                    for (int k = 0; k < 3; ++k) rgb[k] = hor[k] + (zen[k] - hor[k]) * t;
                } else {
                    double t = std::min(1.0, -d[1] * 4.0);
                    for (int k = 0; k < 3; ++k) rgb[k] = hor[k] * 0.6 + (gnd[k] - hor[k] * 0.6) * t;
                }
                double cs = d[0] * own->sun.direction[0] + d[1] * own->sun.direction[1] + d[2] * own->sun.direction[2];
                double glow = cs > 0.0 ? 8.0 * std::pow(cs, 256.0) + 0.6 * std::pow(cs, 8.0) : 0.0;
                uint16_t* t = &own->sky[((size_t)i * W + j) * 4];
                for (int k = 0; k < 3; ++k) t[k] = float_to_half((float)(rgb[k] + glow));
                t[3] = float_to_half(1.0f);
            }
        }
        sky.kind = BSM_SKY_EQUIRECT;
        sky.color[0] = sky.color[1] = sky.color[2] = 1.0f;
        sky.width = W; sky.height = H;
        if (cam) {
            const float pos[3] = {0.5f, 0.55f, 0.0f};
            const float tgt[3] = {0.5f, 0.0f, 0.46f};
            double f[3] = {tgt[0] - pos[0], tgt[1] - pos[1], tgt[2] - pos[2]};
            normalize3(f);
            for (int i = 0; i < 3; ++i) { cam->position[i] = pos[i]; cam->front[i] = (float)f[i]; }
            cam->up[0] = 0; cam->up[1] = 1; cam->up[2] = 0;
            cam->yfov_deg = 60.0f;
        }
    } else {
        delete own;
        return BSM_ERR_INVALID_ARG;
    }
    own->pos.swap(b.pos);
    own->idx.swap(b.idx);
    own->mat.swap(b.mat);
    own->mats.swap(b.mats);
    std::memset(desc, 0, sizeof(*desc));
    desc->num_vertices = (uint32_t)(own->pos.size() / 3);
    desc->positions = own->pos.data();
    desc->num_triangles = (uint32_t)(own->idx.size() / 3);
    desc->indices = own->idx.data();
    desc->material_ids = own->mat.data();
    desc->num_materials = (uint32_t)own->mats.size();
    desc->materials = own->mats.data();
    desc->num_dir_lights = 1;
    desc->dir_lights = &own->sun;
    sky.rgba16f = own->sky.empty() ? nullptr : own->sky.data();
    desc->sky = sky;
    std::lock_guard<std::mutex> lk(g_owned_mu);
    g_owned[desc->positions] = own;
    return BSM_OK;
}

extern "C" void bsm_scene_gen_free(bsm_scene_desc* desc) {
    if (!desc || !desc->positions) return;
    Owned* own = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_owned_mu);
        auto it = g_owned.find(desc->positions);
        if (it == g_owned.end()) return;
        own = it->second;
        g_owned.erase(it);
    }
    delete own;
    std::memset(desc, 0, sizeof(*desc));
}
