// scene.cpp — Scene::createGLContext for CUDA: flattening, light and
// environment sampling tables, Sobol matrices, per-pixel seeds, camera
// uniforms, and the device upload (src/core/Scene.cpp:133-270).
#include "scene.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <utility>

#include "zgl_internal.h"
#include "zmath.cuh"

namespace zgl {
namespace {

struct DirNum {
    int s;
    uint32_t a;
    uint32_t m[12];
};
const DirNum kDirNums[255] = {
#include "sobol_dirnums.inc"
};

}  // namespace

// 256 x 32 Sobol generator matrices: dimension 0 is the van der Corput
// sequence, the others follow the Bratley-Fox recurrence of their primitive
// polynomial; column i of a dimension is the direction number V_{i+1}.
void sobol_matrices(std::vector<uint32_t>& out) {
    out.assign(256 * 32, 0u);
    for (int i = 0; i < 32; i++) out[(size_t)i] = 1u << (31 - i);
    for (int d = 1; d < 256; d++) {
        const DirNum& dn = kDirNums[d - 1];
        uint64_t m[32];
        for (int i = 0; i < dn.s; i++) m[i] = dn.m[i];
        for (int i = dn.s; i < 32; i++) {
            uint64_t v = m[i - dn.s] ^ (m[i - dn.s] << dn.s);
            for (int k = 1; k < dn.s; k++)
                if ((dn.a >> (dn.s - 1 - k)) & 1u) v ^= m[i - k] << k;
            m[i] = v;
        }
        for (int i = 0; i < 32; i++) out[(size_t)d * 32 + i] = (uint32_t)((m[i] << (31 - i)) & 0xffffffffu);
    }
}

// float -> binary16 (round to nearest even, overflow to infinity) -> float:
// the value a texel holds after an RGB16F upload.
float half_round(float x) {
    uint32_t u = zf2bits(x);
    uint32_t sign = u & 0x80000000u;
    int exp = (int)((u >> 23) & 0xffu);
    uint32_t mant = u & 0x7fffffu;
    if (exp == 255) return x;
    int e = exp - 127;
    if (e > 15) return zbits2f(sign | 0x7f800000u);
    if (e >= -14) {
        uint32_t keep = mant >> 13, rest = mant & 0x1fffu;
        if (rest > 0x1000u || (rest == 0x1000u && (keep & 1u))) keep++;
        if (keep == 0x400u) {
            keep = 0;
            e++;
            if (e > 15) return zbits2f(sign | 0x7f800000u);
        }
        return zbits2f(sign | ((uint32_t)(e + 127) << 23) | (keep << 13));
    }
    float a = std::fabs(x) * 16777216.0f;  // exact scaling by 2^24
    float q = std::nearbyint(a);           // nearest multiple of 2^-24, ties to even
    float r = q * (1.0f / 16777216.0f);
    return sign ? -r : r;
}

namespace {

// AliasTable::build (src/math/AliasTable.h:12-54).
void alias_build(const std::vector<float>& pdf, std::vector<int32_t>& alias, std::vector<float>& prob) {
    int n = (int)pdf.size();
    alias.assign((size_t)n, 0);
    prob = pdf;
    float sum = 0.0f;
    for (int i = 0; i < n; i++) sum += prob[(size_t)i];
    float sumInv = (float)n / sum;
    std::vector<std::pair<int, float>> greater, lesser;
    greater.reserve((size_t)n);
    lesser.reserve((size_t)n);
    for (int i = 0; i < n; i++) {
        prob[(size_t)i] *= sumInv;
        (prob[(size_t)i] < 1.0f ? lesser : greater).push_back({i, prob[(size_t)i]});
    }
    while (!greater.empty() && !lesser.empty()) {
        auto [l, pl] = lesser.back();
        lesser.pop_back();
        auto [g, pg] = greater.back();
        greater.pop_back();
        alias[(size_t)l] = g;
        prob[(size_t)l] = pl;
        pg += pl - 1.0f;
        (pg < 1.0f ? lesser : greater).push_back({g, pg});
    }
    while (!greater.empty()) {
        auto [g, pg] = greater.back();
        greater.pop_back();
        alias[(size_t)g] = g;
        prob[(size_t)g] = pg;
    }
    while (!lesser.empty()) {
        auto [l, pl] = lesser.back();
        lesser.pop_back();
        alias[(size_t)l] = l;
        prob[(size_t)l] = pl;
    }
}

// EnvironmentMap::setupAliasTable (EnvironmentMap.cpp:66-114): leftover
// entries get probability 1, the pdf sum is returned.
float env_alias(int32_t* alias, float* pdf, int n, int stride) {
    float sum = 0.0f;
    for (int i = 0, o = 0; i < n; i++, o += stride) sum += pdf[o];
    float sumInv = (float)n / sum;
    std::vector<std::pair<int, float>> greater, lesser;
    for (int i = 0, o = 0; i < n; i++, o += stride) {
        pdf[o] *= sumInv;
        (pdf[o] < 1.0f ? lesser : greater).push_back({i, pdf[o]});
    }
    while (!greater.empty() && !lesser.empty()) {
        auto [l, pl] = lesser.back();
        lesser.pop_back();
        auto [g, pg] = greater.back();
        greater.pop_back();
        alias[l * stride] = g;
        pdf[l * stride] = pl;
        pg += pl - 1.0f;
        (pg < 1.0f ? lesser : greater).push_back({g, pg});
    }
    while (!greater.empty()) {
        int g = greater.back().first;
        greater.pop_back();
        alias[g * stride] = g;
        pdf[g * stride] = 1.0f;
    }
    while (!lesser.empty()) {
        int l = lesser.back().first;
        lesser.pop_back();
        alias[l * stride] = l;
        pdf[l * stride] = 1.0f;
    }
    return sum;
}

// glm::normalize: x * inversesqrt(dot(x, x))
v3 glm_normalize(v3 v) { return v * (1.0f / std::sqrt(dot(v, v))); }

void camera_update(zgl_scene& s, const float* angle, float fov) {  // Camera.cpp:149-162
    const float rad = 0.01745329251994329576923690768489f;  // glm::radians
    float ax = angle[0] * rad, ay = angle[1] * rad;
    float x = std::sin(ax) * std::cos(ay);
    float y = std::cos(ax) * std::cos(ay);
    float z = std::sin(ay);
    v3 front = glm_normalize(mk3(x, y, z));
    v3 right = glm_normalize(cross(front, mk3(0.0f, 0.0f, 1.0f)));
    // glm::rotate(mat4(1), angle.z, front): Rodrigues rotation about the unit
    // axis; the reference passes the roll value straight through as radians.
    float c = std::cos(angle[2]), sn = std::sin(angle[2]);
    v3 axis = glm_normalize(front);
    v3 temp = axis * (1.0f - c);
    float R00 = c + temp.x * axis.x, R01 = temp.x * axis.y + sn * axis.z, R02 = temp.x * axis.z - sn * axis.y;
    float R10 = temp.y * axis.x - sn * axis.z, R11 = c + temp.y * axis.y, R12 = temp.y * axis.z + sn * axis.x;
    float R20 = temp.z * axis.x + sn * axis.y, R21 = temp.z * axis.y - sn * axis.x, R22 = c + temp.z * axis.z;
    v3 rr = mk3((R00 * right.x + R10 * right.y) + R20 * right.z, (R01 * right.x + R11 * right.y) + R21 * right.z,
                (R02 * right.x + R12 * right.y) + R22 * right.z);
    right = glm_normalize(rr);
    v3 up = glm_normalize(cross(right, front));
    m3 inv = inverse(m3{right, up, front});
    s.camF[0] = front.x; s.camF[1] = front.y; s.camF[2] = front.z;
    s.camR[0] = right.x; s.camR[1] = right.y; s.camR[2] = right.z;
    s.camU[0] = up.x; s.camU[1] = up.y; s.camU[2] = up.z;
    float m[9] = {inv.c0.x, inv.c0.y, inv.c0.z, inv.c1.x, inv.c1.y, inv.c1.z, inv.c2.x, inv.c2.y, inv.c2.z};
    std::memcpy(s.camMatInv, m, sizeof(m));
    s.tanFOV = std::tan(fov * 0.5f * rad);
}

// Runs f(b, e) over [0, n) in contiguous chunks of at least `grain` items on
// the host threads (inline when n is small).  f must not throw.
template <class F>
void parallel_for(int64_t n, F&& f, int64_t grain = 4096) {
    const int nt = (int)std::min<int64_t>(host_threads(), std::max<int64_t>(1, n / grain));
    if (nt <= 1) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    const int64_t chunk = (n + nt - 1) / nt;
    for (int t = 0; t < nt; t++) {
        const int64_t b = t * chunk, e = std::min(n, b + chunk);
        if (b < e) th.emplace_back([&f, b, e] { f(b, e); });
    }
    for (auto& x : th) x.join();
}

// Smallest i in [0, n) with bad(i), or -1; checked on the host threads.
template <class P>
int64_t first_bad(int64_t n, P&& bad) {
    std::atomic<int64_t> first{INT64_MAX};
    parallel_for(n, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++)
            if (bad(i)) {
                int64_t cur = first.load();
                while (i < cur && !first.compare_exchange_weak(cur, i)) {
                }
                return;
            }
    }, 1 << 16);
    const int64_t f = first.load();
    return f == INT64_MAX ? -1 : f;
}

// libstdc++'s std::default_random_engine (minstd_rand0, seed 1) through
// uniform_real_distribution<float>(0, 1): Sampler::genNoiseTexture
// (Sampler.cpp:66-80) as built by GCC.
// The draws are split over host threads; each chunk starts from the
// engine's state at its first index (16807^i mod (2^31 - 1)), so the values
// equal the sequential stream.
void noise_texture(int W, int H, std::vector<float>& out) {
    out.resize((size_t)W * H * 2);
    const uint64_t p = 2147483647u;
    parallel_for((int64_t)out.size(), [&](int64_t b, int64_t e) {
        uint64_t x = 1, base = 16807u;
        for (uint64_t k = (uint64_t)b; k; k >>= 1) {  // x = 16807^b mod p
            if (k & 1u) x = (x * base) % p;
            base = (base * base) % p;
        }
        for (int64_t i = b; i < e; i++) {
            x = (x * 16807u) % p;
            float v = (float)(x - 1) / 2147483646.0f;
            if (v >= 1.0f) v = std::nextafter(1.0f, 0.0f);
            out[(size_t)i] = v * (1.0f - 0.0f) + 0.0f;
        }
    });
}

// texture(uNoiseTex, st): bilinear, repeat wrap, texel centres at (i + 0.5) / size.
v2 noise_lookup(const std::vector<float>& t, int W, int H, v2 st) {
    auto tex = [&](int x, int y) {
        x %= W;
        if (x < 0) x += W;
        y %= H;
        if (y < 0) y += H;
        const float* p = &t[2 * ((size_t)y * W + x)];
        return mk2(p[0], p[1]);
    };
    float u = st.x * (float)W - 0.5f, v = st.y * (float)H - 0.5f;
    float fu = std::floor(u), fv = std::floor(v);
    float au = u - fu, av = v - fv;
    int x0 = zf2i(fu), y0 = zf2i(fv);
    v2 t00 = tex(x0, y0), t10 = tex(x0 + 1, y0), t01 = tex(x0, y0 + 1), t11 = tex(x0 + 1, y0 + 1);
    auto mix2 = [](v2 a, v2 b, float k) { return mk2(a.x * (1.0f - k) + b.x * k, a.y * (1.0f - k) + b.y * k); };
    return mix2(mix2(t00, t10, au), mix2(t01, t11, au), av);
}

// Per-pixel seed factors of path_integ_naive.glsl:156-160:
// noiseCoord = tex(noise, tex(noise, coord / size)); (uint(W n.x), uint(H n.y)).
void pixel_seeds(const std::vector<float>& noise, int W, int H, std::vector<uint32_t>& out) {
    out.resize((size_t)W * H * 2);
    const v2 size = mk2((float)W, (float)H);
    parallel_for(H, [&](int64_t y0, int64_t y1) {
        for (int y = (int)y0; y < (int)y1; y++)
            for (int x = 0; x < W; x++) {
                v2 scr = mk2((float)x, (float)y) / size;
                v2 nc = noise_lookup(noise, W, H, scr);
                nc = noise_lookup(noise, W, H, nc);
                v2 tc = size * nc;
                out[2 * ((size_t)y * W + x)] = zf2u(tc.x);
                out[2 * ((size_t)y * W + x) + 1] = zf2u(tc.y);
            }
    }, 8);
}

template <class T>
T* upload(const std::vector<T>& v) {
    if (v.empty()) return nullptr;
    T* d = nullptr;
    ZGL_CUDA(cudaMalloc(&d, sizeof(T) * v.size()));
    ZGL_CUDA(cudaMemcpy(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
    return d;
}

// Per-triangle light power (instance power split by area), light areas, the
// light alias table and the power sum (Scene.cpp:200-243).  Light triangle t
// is scene triangle objPrimCount + t.
void light_tables(zgl_scene& s) {
    std::vector<float> pdf;
    s.lightPower.clear();
    s.lightArea.clear();
    s.lightAlias.clear();
    s.lightProb.clear();
    s.lightSum = 0.0f;
    auto vert = [&](uint32_t t, int j) {
        const float* p = &s.vertices[3 * (size_t)s.indices[3 * ((size_t)s.objPrimCount + t) + j]];
        return mk3(p[0], p[1], p[2]);
    };
    for (size_t k = 0; k + 1 < s.lightFirst.size(); k++) {
        uint32_t f0 = s.lightFirst[k], f1 = s.lightFirst[k + 1];
        v3 P = mk3(s.lightInstPower[3 * k], s.lightInstPower[3 * k + 1], s.lightInstPower[3 * k + 2]);
        float sumArea = 0.0f;
        for (uint32_t t = f0; t < f1; t++) sumArea += length(cross(vert(t, 2) - vert(t, 0), vert(t, 1) - vert(t, 0)));
        for (uint32_t t = f0; t < f1; t++) {
            v3 a = vert(t, 0), b = vert(t, 1), c = vert(t, 2);
            float area = length(cross(c - a, b - a));
            v3 pw = P * area / sumArea;
            s.lightPower.push_back(pw.x);
            s.lightPower.push_back(pw.y);
            s.lightPower.push_back(pw.z);
            s.lightArea.push_back(0.5f * length(cross(c - a, b - a)));  // triangleArea (math.glsl:147-150)
            float l = dot(pw, mk3(0.299f, 0.587f, 0.114f));
            pdf.push_back(l);
            s.lightSum += l;
        }
    }
    if (!pdf.empty()) alias_build(pdf, s.lightAlias, s.lightProb);
    if (s.nLight > 0 && !(s.lightSum > 0.0f))
        fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: lights have zero total power or zero area");
}

// sRGB code -> linear value (the sRGB transfer function of GL_SRGB textures,
// evaluated in double and rounded once to float)
void srgb_lut(std::vector<float>& lut) {
    lut.resize(256);
    for (int i = 0; i < 256; i++) {
        double c = i / 255.0;
        lut[(size_t)i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
    }
}

// Texture2DArray (Texture.cpp:134-171): layers of the largest width and
// height, each image in the top-left corner of its layer (the rest zero),
// uv scale = image size / layer size; and the object texcoords.
void texture_tables(zgl_scene& s, const zgl_scene_desc& d) {
    const size_t nvo = d.obj_n_vertices;
    s.texcoords.assign(2 * nvo, 0.0f);
    if (d.obj_texcoords) {
        s.texcoords.assign(d.obj_texcoords, d.obj_texcoords + 2 * nvo);
        for (float x : s.texcoords)
            if (!std::isfinite(x)) fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: texcoord not finite");
    }
    if (d.n_textures < 0 || d.n_textures > 0x7fff)
        fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: %d textures (0..32767)", d.n_textures);
    s.nTextures = d.n_textures;
    s.texMaxW = s.texMaxH = 0;
    s.texels.clear();
    s.texScale.clear();
    srgb_lut(s.srgbLut);
    if (s.nTextures == 0) return;
    if (!d.tex_size || !d.tex_rgb) fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: textures need tex_size and tex_rgb");
    for (int t = 0; t < s.nTextures; t++) {
        int32_t w = d.tex_size[2 * t], h = d.tex_size[2 * t + 1];
        if (w <= 0 || h <= 0 || w > 16384 || h > 16384)
            fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: texture %d size %dx%d out of range", t, w, h);
        s.texMaxW = std::max(s.texMaxW, w);
        s.texMaxH = std::max(s.texMaxH, h);
    }
    const size_t layer = (size_t)s.texMaxW * s.texMaxH;
    if (layer * (size_t)s.nTextures > ((size_t)1 << 31))
        fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: texture array above 2^31 texels");
    s.texels.assign(layer * (size_t)s.nTextures, 0u);
    s.texScale.resize(2 * (size_t)s.nTextures);
    const uint8_t* src = d.tex_rgb;
    for (int t = 0; t < s.nTextures; t++) {
        int32_t w = d.tex_size[2 * t], h = d.tex_size[2 * t + 1];
        uint32_t* dst = &s.texels[layer * (size_t)t];
        for (int32_t y = 0; y < h; y++)
            for (int32_t x = 0; x < w; x++, src += 3)
                dst[(size_t)y * s.texMaxW + x] = (uint32_t)src[0] | ((uint32_t)src[1] << 8) | ((uint32_t)src[2] << 16);
        s.texScale[2 * (size_t)t] = (float)w / (float)s.texMaxW;
        s.texScale[2 * (size_t)t + 1] = (float)h / (float)s.texMaxH;
    }
}

void build_scene(zgl_scene& s, const zgl_scene_desc& d) {
    if (d.obj_n_triangles > 0 && (!d.obj_vertices || !d.obj_normals || !d.obj_indices || !d.obj_mat_tex))
        fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: object arrays missing");
    if (d.light_n_triangles > 0 && (!d.light_vertices || !d.light_normals || !d.light_indices))
        fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: light arrays missing");
    if (d.n_light_instances > 0 && (!d.light_first || !d.light_power))
        fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: light instances need light_first and light_power");
    if (d.film_width <= 0 || d.film_height <= 0 || d.film_width > 16384 || d.film_height > 16384)
        fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: film size %dx%d out of range", d.film_width, d.film_height);
    if (d.sampler != 0 && d.sampler != 1) fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: sampler must be 0 or 1");
    if (d.obj_n_triangles + d.light_n_triangles > (size_t)0x3fffffff)
        fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: too many triangles");
    if (d.n_materials > 0xffff) fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: more than 65535 materials");
    if (d.obj_n_triangles > 0 && d.n_materials == 0)
        fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: object triangles need materials");

    // flatten: objects first, then lights
    size_t nvo = d.obj_n_vertices, nvl = d.light_n_vertices;
    s.vertices.assign(d.obj_vertices, d.obj_vertices + 3 * nvo);
    s.normals.assign(d.obj_normals, d.obj_normals + 3 * nvo);
    if (nvl) {
        s.vertices.insert(s.vertices.end(), d.light_vertices, d.light_vertices + 3 * nvl);
        s.normals.insert(s.normals.end(), d.light_normals, d.light_normals + 3 * nvl);
    }
    if (first_bad((int64_t)s.vertices.size(), [&](int64_t i) { return !(s.vertices[(size_t)i] == s.vertices[(size_t)i]); }) >= 0)
        fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: NaN vertex coordinate");
    s.indices.assign(d.obj_indices, d.obj_indices + 3 * d.obj_n_triangles);
    {
        const int64_t i = first_bad(3 * (int64_t)d.obj_n_triangles, [&](int64_t k) { return d.obj_indices[k] >= nvo; });
        if (i >= 0) fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: object index %lld out of range", (long long)i);
    }
    for (size_t i = 0; i < 3 * d.light_n_triangles; i++) {
        if (d.light_indices[i] >= nvl) fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: light index %zu out of range", i);
        s.indices.push_back((uint32_t)(d.light_indices[i] + nvo));
    }
    s.objPrimCount = (int32_t)d.obj_n_triangles;
    s.nObjVertices = (int64_t)nvo;
    s.nLight = (int32_t)d.light_n_triangles;
    s.ntri = (int64_t)(d.obj_n_triangles + d.light_n_triangles);

    // materials and per-triangle material indices
    s.materials.assign(d.materials, d.materials + 16 * d.n_materials);
    for (size_t m = 0; m < d.n_materials; m++) {
        int32_t type;
        std::memcpy(&type, &s.materials[16 * m + 13], 4);
        if (type < 0 || type > 4)
            fail(ZGL_ERR_INVALID_ARG,
                 "zgl_scene_create: material %zu has type %d; the types are lambertian (0), principled (1), "
                 "metal workflow (2), dielectric (3) and thin dielectric (4)", m, type);
        if ((type == 3 || type == 4) && !(s.materials[16 * m + 12] > 0.0f))
            fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: dielectric material %zu needs ior > 0", m);
        if (type >= 2) s.fullMaterials = true;
        for (int k = 0; k < 13; k++)
            if (!std::isfinite(s.materials[16 * m + k]))
                fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: material %zu parameter %d is not finite", m, k);
    }
    texture_tables(s, d);
    s.matTex.assign(d.obj_mat_tex, d.obj_mat_tex + d.obj_n_triangles);
    {
        const int64_t t = first_bad((int64_t)d.obj_n_triangles, [&](int64_t k) {
            const int32_t mt = s.matTex[(size_t)k], mat = mt & 0xffff, tex = mt >> 16;
            return (tex != -1 && (tex < 0 || tex >= s.nTextures)) || (size_t)mat >= d.n_materials;
        });
        if (t >= 0) {
            const int32_t tex = s.matTex[(size_t)t] >> 16;
            if (tex != -1 && (tex < 0 || tex >= s.nTextures))
                fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: triangle %lld uses texture %d of %d", (long long)t, tex,
                     s.nTextures);
            fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: triangle %lld material out of range", (long long)t);
        }
        // a textured triangle selects the full material instantiation
        if (s.nTextures > 0 &&
            first_bad((int64_t)d.obj_n_triangles, [&](int64_t k) { return (s.matTex[(size_t)k] >> 16) != -1; }) >= 0)
            s.fullMaterials = true;
    }

    // light instances, then power split by area and the light alias table
    size_t covered = 0;
    s.lightFirst.assign(1, 0u);
    for (size_t k = 0; k < d.n_light_instances; k++) {
        uint32_t f0 = d.light_first[k], f1 = d.light_first[k + 1];
        if (f0 != covered || f1 < f0 || f1 > d.light_n_triangles)
            fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: light_first must partition the light triangles");
        covered = f1;
        s.lightFirst.push_back(f1);
        for (int c = 0; c < 3; c++) s.lightInstPower.push_back(d.light_power[3 * k + c]);
    }
    if (covered != d.light_n_triangles)
        fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: light_first does not cover every light triangle");
    light_tables(s);

    // environment map (EnvironmentMap.cpp:8-59)
    s.envRotation = d.env_rotation;
    if (d.env_rgb) {
        int W = d.env_width, H = d.env_height;
        if (W <= 0 || H <= 0 || (int64_t)W * H > (1ll << 28))
            fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: bad environment size %dx%d", W, H);
        s.envW = W;
        s.envH = H;
        size_t n = (size_t)W * H * 3;
        s.envTexels.resize(n);
        std::atomic<bool> bad{false};
        parallel_for((int64_t)n, [&](int64_t b, int64_t e) {
            for (int64_t i = b; i < e; i++) {
                float v = d.env_rgb[i];
                if (!std::isfinite(v) || v < 0.0f) bad = true;
                s.envTexels[(size_t)i] = half_round(v);
            }
        });
        if (bad) fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: bad environment texel");
        s.envAlias.assign((size_t)(W + 1) * H, 0);
        s.envProb.assign((size_t)(W + 1) * H, 0.0f);
        auto off = [W](int i, int j) { return (size_t)i * (W + 1) + j; };
        // per row: luminance times the row's solid-angle weight, then the
        // row's alias table (rows are independent)
        parallel_for(H, [&](int64_t r0, int64_t r1) {
            for (int i = (int)r0; i < (int)r1; i++) {
                for (int j = 0; j < W; j++) {
                    const float* p = d.env_rgb + 3 * ((size_t)i * W + j);
                    float lum = 0.2126f * p[0] + 0.7152f * p[1] + 0.0722f * p[2];
                    s.envProb[off(i, j)] = lum * std::sin((float)(i + 0.5f) / (float)H * 3.141592653589793f);
                }
                s.envProb[off(i, W)] = env_alias(&s.envAlias[off(i, 0)], &s.envProb[off(i, 0)], W, 1);
            }
        }, 8);
        float sum = env_alias(&s.envAlias[(size_t)W], &s.envProb[(size_t)W], H, W + 1);
        s.envSum = (float)zf2i(sum);  // EnvironmentMap::sumPdf returns int
    }

    // sampler tables (Sampler.cpp:48-80)
    s.sampler = d.sampler;
    s.filmW = d.film_width;
    s.filmH = d.film_height;
    sobol_matrices(s.sobol);
    noise_texture(s.filmW, s.filmH, s.noise);
    pixel_seeds(s.noise, s.filmW, s.filmH, s.seeds);

    // camera (Scene.cpp:86-103)
    float fov = d.cam_fov;
    if (fov > 90.0f) fov = 90.0f;
    if (fov < 0.1f) fov = 0.1f;
    std::memcpy(s.camPos, d.cam_pos, sizeof(s.camPos));
    camera_update(s, d.cam_angle, fov);
    s.camAsp = (float)s.filmW / (float)s.filmH;
    s.lensRadius = d.cam_lens_radius;
    s.focalDist = d.cam_focal_dist;
}

void upload_scene(zgl_scene& s) {
    ZGL_CUDA(cudaGetDevice(&s.device));
    // the CUDA builder: the same PackedBVH as the host builder, bit for bit
    s.accel = accel_create_device(s.vertices.data(), (int64_t)s.vertices.size() / 3, s.indices.data(), s.ntri, 0,
                                  0);
    std::vector<float4> shade((size_t)s.ntri * 5);
    parallel_for(s.ntri, [&](int64_t t0, int64_t t1) {
        for (int64_t t = t0; t < t1; t++) {
            auto P = [&](int j) { return &s.vertices[3 * (size_t)s.indices[3 * t + j]]; };
            auto N = [&](int j) { return &s.normals[3 * (size_t)s.indices[3 * t + j]]; };
            const float *a = P(0), *b = P(1), *c = P(2), *na = N(0), *nb = N(1), *nc = N(2);
            int32_t mt = t < s.objPrimCount ? s.matTex[(size_t)t] : -1;
            float mtf;
            std::memcpy(&mtf, &mt, 4);
            shade[5 * t + 0] = make_float4(a[0], a[1], a[2], b[0]);
            shade[5 * t + 1] = make_float4(b[1], b[2], c[0], c[1]);
            shade[5 * t + 2] = make_float4(c[2], na[0], na[1], na[2]);
            shade[5 * t + 3] = make_float4(nb[0], nb[1], nb[2], nc[0]);
            shade[5 * t + 4] = make_float4(nc[1], nc[2], mtf, 0.0f);
        }
    });
    s.d_shade = upload(shade);
    std::vector<float4> mats(s.materials.size() / 4);
    for (size_t i = 0; i < mats.size(); i++)
        mats[i] = make_float4(s.materials[4 * i], s.materials[4 * i + 1], s.materials[4 * i + 2], s.materials[4 * i + 3]);
    s.d_materials = upload(mats);
    std::vector<float4> lp((size_t)s.nLight);
    for (int i = 0; i < s.nLight; i++)
        lp[(size_t)i] = make_float4(s.lightPower[3 * i], s.lightPower[3 * i + 1], s.lightPower[3 * i + 2], s.lightArea[(size_t)i]);
    s.d_lightPower = upload(lp);
    s.d_lightAlias = upload(s.lightAlias);
    s.d_lightProb = upload(s.lightProb);
    if (!s.envTexels.empty()) {
        std::vector<float4> env((size_t)s.envW * s.envH);
        for (size_t i = 0; i < env.size(); i++)
            env[i] = make_float4(s.envTexels[3 * i], s.envTexels[3 * i + 1], s.envTexels[3 * i + 2], 0.0f);
        s.d_env = upload(env);
        s.d_envAlias = upload(s.envAlias);
        s.d_envProb = upload(s.envProb);
    }
    s.d_sobol = upload(s.sobol);
    std::vector<uint2> seeds((size_t)s.filmW * s.filmH);
    for (size_t i = 0; i < seeds.size(); i++) seeds[i] = make_uint2(s.seeds[2 * i], s.seeds[2 * i + 1]);
    s.d_seeds = upload(seeds);
    if (s.nTextures > 0) {
        std::vector<float2> uv((size_t)s.objPrimCount * 3);
        for (size_t i = 0; i < uv.size(); i++) {
            uint32_t vi = s.indices[i];
            uv[i] = make_float2(s.texcoords[2 * (size_t)vi], s.texcoords[2 * (size_t)vi + 1]);
        }
        s.d_uv = upload(uv);
        s.d_texels = upload(s.texels);
        std::vector<float2> sc((size_t)s.nTextures);
        for (size_t t = 0; t < sc.size(); t++) sc[t] = make_float2(s.texScale[2 * t], s.texScale[2 * t + 1]);
        s.d_texScale = upload(sc);
        s.d_srgb = upload(s.srgbLut);
    }
}

}  // namespace

// Writes new material parameters (per material: baseColor rgb, roughness,
// metallic, specular into record slots 0-3, 5, 6) and light-instance powers
// (3 per instance), rebuilds the light tables that depend on the powers and
// updates the device copies in place.
void scene_set_diff_params(zgl_scene* s, const float* p, int nmat, std::vector<float>& instPower) {
    const int ninst = (int)(instPower.size() / 3);
    for (int k = 0; k < 3 * ninst; k++)
        if (p[6 * nmat + k] < 0.0f) fail(ZGL_ERR_INVALID_ARG, "zgl_diff_set_params: negative light power");
    std::vector<float> oldInst = s->lightInstPower;
    for (int k = 0; k < 3 * ninst; k++) s->lightInstPower[(size_t)k] = p[6 * nmat + k];
    try {
        light_tables(*s);
    } catch (...) {
        s->lightInstPower = oldInst;
        light_tables(*s);
        throw;
    }
    instPower = s->lightInstPower;
    for (int m = 0; m < nmat; m++) {
        float* r = &s->materials[16 * (size_t)m];
        const float* q = p + 6 * (size_t)m;
        r[0] = q[0];
        r[1] = q[1];
        r[2] = q[2];
        r[3] = q[3];
        r[5] = q[4];
        r[6] = q[5];
    }
    if (nmat > 0)
        ZGL_CUDA(cudaMemcpy(s->d_materials, s->materials.data(), sizeof(float) * s->materials.size(),
                            cudaMemcpyHostToDevice));
    if (s->nLight > 0) {
        std::vector<float4> lp((size_t)s->nLight);
        for (int i = 0; i < s->nLight; i++)
            lp[(size_t)i] = make_float4(s->lightPower[3 * i], s->lightPower[3 * i + 1], s->lightPower[3 * i + 2],
                                        s->lightArea[(size_t)i]);
        ZGL_CUDA(cudaMemcpy(s->d_lightPower, lp.data(), sizeof(float4) * lp.size(), cudaMemcpyHostToDevice));
        ZGL_CUDA(cudaMemcpy(s->d_lightAlias, s->lightAlias.data(), 4 * s->lightAlias.size(), cudaMemcpyHostToDevice));
        ZGL_CUDA(cudaMemcpy(s->d_lightProb, s->lightProb.data(), 4 * s->lightProb.size(), cudaMemcpyHostToDevice));
    }
}

}  // namespace zgl

zgl::DeviceScene zgl_scene::view() const {
    zgl::DeviceScene v{};
    v.accel = zgl::device_view(accel);
    v.shade = d_shade;
    v.materials = d_materials;
    v.objPrimCount = objPrimCount;
    v.nLight = nLight;
    v.lightPower = d_lightPower;
    v.lightAlias = d_lightAlias;
    v.lightProb = d_lightProb;
    v.lightSum = lightSum;
    v.envTexels = d_env;
    v.envW = envW;
    v.envH = envH;
    v.envAlias = d_envAlias;
    v.envProb = d_envProb;
    v.envSum = envSum;
    v.envRotation = envRotation;
    v.sobol = d_sobol;
    v.pixelSeeds = d_seeds;
    v.sampler = sampler;
    v.camF = make_float3(camF[0], camF[1], camF[2]);
    v.camR = make_float3(camR[0], camR[1], camR[2]);
    v.camU = make_float3(camU[0], camU[1], camU[2]);
    v.camPos = make_float3(camPos[0], camPos[1], camPos[2]);
    std::memcpy(v.camMatInv, camMatInv, sizeof(camMatInv));
    v.tanFOV = tanFOV;
    v.lensRadius = lensRadius;
    v.focalDist = focalDist;
    v.camAsp = camAsp;
    v.filmW = filmW;
    v.filmH = filmH;
    v.uv = d_uv;
    v.texels = d_texels;
    v.texScale = d_texScale;
    v.srgb = d_srgb;
    v.texW = texMaxW;
    v.texH = texMaxH;
    return v;
}

void zgl_scene::free_device() {
    zgl::accel_free(accel);
    accel = nullptr;
    for (void* p : {(void*)d_shade, (void*)d_materials, (void*)d_lightPower, (void*)d_lightAlias, (void*)d_lightProb,
                    (void*)d_env, (void*)d_envAlias, (void*)d_envProb, (void*)d_sobol, (void*)d_seeds,
                    (void*)d_uv, (void*)d_texels, (void*)d_texScale, (void*)d_srgb})
        if (p) cudaFree(p);
    d_uv = nullptr;
    d_texels = nullptr;
    d_texScale = nullptr;
    d_srgb = nullptr;
    d_shade = d_materials = d_lightPower = d_env = nullptr;
    d_lightAlias = d_envAlias = nullptr;
    d_lightProb = d_envProb = nullptr;
    d_sobol = nullptr;
    d_seeds = nullptr;
}

using namespace zgl;

extern "C" {

zgl_status zgl_scene_create(const zgl_scene_desc* desc, int32_t flags, zgl_scene** out) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_scene_create");
    if (!desc || !out) fail(ZGL_ERR_INVALID_ARG, "zgl_scene_create: NULL argument");
    *out = nullptr;
    auto* s = new zgl_scene();
    try {
        build_scene(*s, *desc);
        s->host_only = (flags & ZGL_SCENE_HOST_ONLY) != 0;
        if (!s->host_only) upload_scene(*s);
    } catch (...) {
        s->free_device();
        delete s;
        throw;
    }
    *out = s;
    ZGL_API_END
}

zgl_status zgl_scene_export(const zgl_scene* s, const char* table, void* out, size_t bytes) {
    ZGL_API_BEGIN
    if (!s || !table || !out) fail(ZGL_ERR_INVALID_ARG, "zgl_scene_export: NULL argument");
    std::string t(table);
    auto give = [&](const void* src, size_t n) {
        if (n != bytes) fail(ZGL_ERR_INVALID_ARG, "zgl_scene_export: table %s has %zu bytes, %zu given", table, n, bytes);
        if (n) std::memcpy(out, src, n);
    };
    if (t == "light_power") give(s->lightPower.data(), 4 * s->lightPower.size());
    else if (t == "light_alias") give(s->lightAlias.data(), 4 * s->lightAlias.size());
    else if (t == "light_prob") give(s->lightProb.data(), 4 * s->lightProb.size());
    else if (t == "env_alias") give(s->envAlias.data(), 4 * s->envAlias.size());
    else if (t == "env_prob") give(s->envProb.data(), 4 * s->envProb.size());
    else if (t == "env_texels") give(s->envTexels.data(), 4 * s->envTexels.size());
    else if (t == "sobol") give(s->sobol.data(), 4 * s->sobol.size());
    else if (t == "noise") give(s->noise.data(), 4 * s->noise.size());
    else if (t == "pixel_seeds") give(s->seeds.data(), 4 * s->seeds.size());
    else if (t == "camera") {
        float c[19];
        std::memcpy(c, s->camF, 12);
        std::memcpy(c + 3, s->camR, 12);
        std::memcpy(c + 6, s->camU, 12);
        std::memcpy(c + 9, s->camMatInv, 36);
        c[18] = s->tanFOV;
        give(c, sizeof(c));
    } else if (t == "info") {
        int64_t c[13] = {s->filmW, s->filmH, (int64_t)s->vertices.size() / 3, s->nObjVertices, s->ntri,
                         s->objPrimCount, s->nLight, (int64_t)s->materials.size() / 16, s->envW, s->envH,
                         s->nTextures, s->texMaxW, s->texMaxH};
        give(c, sizeof(c));
    } else if (t == "vertices") give(s->vertices.data(), 4 * s->vertices.size());
    else if (t == "normals") give(s->normals.data(), 4 * s->normals.size());
    else if (t == "indices") give(s->indices.data(), 4 * s->indices.size());
    else if (t == "mat_tex") give(s->matTex.data(), 4 * s->matTex.size());
    else if (t == "materials") give(s->materials.data(), 4 * s->materials.size());
    else if (t == "tex_scale") give(s->texScale.data(), 4 * s->texScale.size());
    else if (t == "texcoords") give(s->texcoords.data(), 4 * s->texcoords.size());
    else if (t == "tex_texels") give(s->texels.data(), 4 * s->texels.size());
    else if (t == "srgb_lut") give(s->srgbLut.data(), 4 * s->srgbLut.size());
    else if (t == "scalars") {
        float c[4] = {s->lightSum, s->envSum, (float)s->objPrimCount, (float)s->nLight};
        give(c, sizeof(c));
    } else fail(ZGL_ERR_INVALID_ARG, "zgl_scene_export: unknown table '%s'", table);
    ZGL_API_END
}

zgl_status zgl_alias_table_build(const float* pdf, size_t n, int32_t* alias, float* prob) {
    ZGL_API_BEGIN
    if (n == 0) return ZGL_OK;
    if (!pdf || !alias || !prob) fail(ZGL_ERR_INVALID_ARG, "zgl_alias_table_build: NULL argument");
    if (n > (size_t)0x7fffffff) fail(ZGL_ERR_INVALID_ARG, "zgl_alias_table_build: n too large");
    std::vector<float> p(pdf, pdf + n);
    std::vector<int32_t> a;
    std::vector<float> q;
    alias_build(p, a, q);
    std::memcpy(alias, a.data(), 4 * n);
    std::memcpy(prob, q.data(), 4 * n);
    ZGL_API_END
}

zgl_status zgl_scene_destroy(zgl_scene* s) {
    ZGL_API_BEGIN
    if (!s) return ZGL_OK;
    s->free_device();
    delete s;
    ZGL_API_END
}

}  // extern "C"
