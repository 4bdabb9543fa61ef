// Headless terrain ray-marcher: glsl/rendering.glsl:1-539 (Render::Data::dispatch,
// src/rendering.cpp:79-140) as CUDA kernels writing an RGBA8 image to device
// memory instead of a GL texture.
//
//   k_pack_heightmap   the world's fields as the shader's heightmap texels
//                      (rock, dirt, water, total = rock + dirt + water) and
//                      the sediment texels (rock, dirt), one float4 / float2
//                      per cell, so a bilinear tap is one 16-byte load
//   k_render           one thread per pixel: primary march on the total
//                      height, water refraction / reflection marches, shadow
//                      march, material shading, fog, sky, gamma
//
// Every operation is a correctly rounded float add, multiply, divide or
// square root in the shader's order (the build has no contraction), except
// pow and exp: GLSL leaves their precision to the driver, so the ray-marcher
// evaluates them with its own exp2 / log2 (below), whose results are the same
// on any IEEE machine.  A CPU restatement with the same exp2 / log2 thus
// renders the same bytes.
#include "hg_internal.h"

#include <cmath>
#include <cstring>

namespace hg {

namespace {

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 scl(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 neg(V3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len(V3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ V3 normalize(V3 a) {
    const float l = len(a);
    return v3(a.x / l, a.y / l, a.z / l);
}
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ V3 mix3(V3 a, V3 b, float t) { return v3(gmix(a.x, b.x, t), gmix(a.y, b.y, t), gmix(a.z, b.z, t)); }
// GLSL reflect(I, N) = I - 2 dot(N, I) N
__device__ __forceinline__ V3 reflect(V3 i, V3 n) { return sub(i, scl(n, 2.0f * dot(n, i))); }
__device__ __forceinline__ float smoothstep(float e0, float e1, float x) {
    const float t = gclamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
__device__ __forceinline__ float fract_(float x) { return x - floorf(x); }

// exp2 by argument reduction to [-1/2, 1/2] and the Taylor series of e^t,
// t = f ln 2, to degree 7 (truncation below 6e-9 relative); 2^n applied as
// two exact power-of-two factors so results down to the subnormal range keep
// their bits.
__device__ __forceinline__ float rm_exp2(float x) {
    if (x != x) return x;
    if (x >= 128.0f) return __int_as_float(0x7f800000);
    if (x < -150.0f) return 0.0f;
    const float n = floorf(x + 0.5f);
    const float f = x - n;
    const float t = f * 0.693147180559945309f;
    float p = 1.0f / 5040.0f;
    p = p * t + 1.0f / 720.0f;
    p = p * t + 1.0f / 120.0f;
    p = p * t + 1.0f / 24.0f;
    p = p * t + 1.0f / 6.0f;
    p = p * t + 0.5f;
    p = p * t + 1.0f;
    p = p * t + 1.0f;
    const int ni = (int)n, a = ni / 2, b = ni - a;
    return p * __int_as_float((a + 127) << 23) * __int_as_float((b + 127) << 23);
}

// log2 of a positive finite x: x = m 2^e with m in [sqrt(1/2), sqrt(2)),
// ln m = 2 atanh(s), s = (m - 1) / (m + 1), |s| < 0.172, by its series to s^9
// (truncation below 1e-9).
__device__ __forceinline__ float rm_log2(float x) {
    int e = 0;
    if (x < 0x1p-126f) {
        x *= 0x1p23f;
        e = -23;
    }
    const uint32_t bits = (uint32_t)__float_as_int(x);
    e += (int)((bits >> 23) & 0xffu) - 127;
    float m = __int_as_float((int)((bits & 0x7fffffu) | 0x3f800000u));
    if (m > 1.41421356f) {
        m *= 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float q = 1.0f / 9.0f;
    q = q * s2 + 1.0f / 7.0f;
    q = q * s2 + 1.0f / 5.0f;
    q = q * s2 + 1.0f / 3.0f;
    q = q * s2 + 1.0f;
    const float ln_m = 2.0f * s * q;
    return (float)e + ln_m * 1.44269504088896341f;
}

// pow(x, y) for the shader's bases: NaN below 0 (GLSL leaves it undefined),
// 0^y = 0 (y > 0) or 1 (y == 0), otherwise exp2(y log2 x)
__device__ __forceinline__ float rm_pow(float x, float y) {
    if (!(x >= 0.0f)) return __int_as_float(0x7fc00000);
    if (x == 0.0f) return y > 0.0f ? 0.0f : (y == 0.0f ? 1.0f : __int_as_float(0x7f800000));
    if (x == __int_as_float(0x7f800000)) return y > 0.0f ? x : (y == 0.0f ? 1.0f : 0.0f);
    return rm_exp2(y * rm_log2(x));
}
__device__ __forceinline__ float rm_exp(float x) { return rm_exp2(x * 1.44269504088896341f); }

constexpr float MAX_DIST = 2048.0f;  // glsl/rendering.glsl:40-41
constexpr int MAX_STEPS = 1024;
constexpr int KIND_TOTAL = 3, KIND_TERRAIN = 4;

struct Scene {
    const float4* hm;  // (rock, dirt, water, total)
    const float2* sed;
    int n;
    float max_height;
    float prec;
    V3 light;  // light_dir = normalize(0, -0.7, 1)
};

struct Materials {
    V3 grass, rock, dirt;
};

__device__ __forceinline__ float4 tex_bilinear(const Scene& S, float px, float py) {
    const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    // every tap is outside the map beyond these bounds (and for NaN)
    if (!(px > -2.0f && px < (float)S.n + 1.0f && py > -2.0f && py < (float)S.n + 1.0f)) return z;
    const int ix = (int)px, iy = (int)py;
    const float fx = fract_(px), fy = fract_(py);
    float4 a, b, c, d;
    if ((unsigned)ix < (unsigned)(S.n - 1) && (unsigned)iy < (unsigned)(S.n - 1)) {  // all four taps inside
        const float4* q = S.hm + (size_t)iy * S.n + ix;
        a = __ldg(q);
        b = __ldg(q + 1);
        c = __ldg(q + S.n);
        d = __ldg(q + S.n + 1);
    } else {
        auto t = [&](int x, int y) {
            return (x >= 0 && x < S.n && y >= 0 && y < S.n) ? __ldg(S.hm + (size_t)y * S.n + x) : z;
        };
        a = t(ix, iy);
        b = t(ix + 1, iy);
        c = t(ix, iy + 1);
        d = t(ix + 1, iy + 1);
    }
    float4 r;
    r.x = gmix(gmix(a.x, b.x, fx), gmix(c.x, d.x, fx), fy);
    r.y = gmix(gmix(a.y, b.y, fx), gmix(c.y, d.y, fx), fy);
    r.z = gmix(gmix(a.z, b.z, fx), gmix(c.z, d.z, fx), fy);
    r.w = gmix(gmix(a.w, b.w, fx), gmix(c.w, d.w, fx), fy);
    return r;
}

// the march's height at (px, py): rock + dirt (terrain rays) or the total
// (primary rays), the same bilinear channels tex_bilinear gives
__device__ __forceinline__ float tex_height(const Scene& S, float px, float py, bool terrain) {
    if (!(px > -2.0f && px < (float)S.n + 1.0f && py > -2.0f && py < (float)S.n + 1.0f))
        return terrain ? 0.0f + 0.0f : 0.0f;
    const int ix = (int)px, iy = (int)py;
    const float fx = fract_(px), fy = fract_(py);
    const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 a, b, c, d;
    if ((unsigned)ix < (unsigned)(S.n - 1) && (unsigned)iy < (unsigned)(S.n - 1)) {
        const float4* q = S.hm + (size_t)iy * S.n + ix;
        a = __ldg(q);
        b = __ldg(q + 1);
        c = __ldg(q + S.n);
        d = __ldg(q + S.n + 1);
    } else {
        auto t = [&](int x, int y) {
            return (x >= 0 && x < S.n && y >= 0 && y < S.n) ? __ldg(S.hm + (size_t)y * S.n + x) : z;
        };
        a = t(ix, iy);
        b = t(ix + 1, iy);
        c = t(ix, iy + 1);
        d = t(ix + 1, iy + 1);
    }
    if (terrain)
        return gmix(gmix(a.x, b.x, fx), gmix(c.x, d.x, fx), fy) + gmix(gmix(a.y, b.y, fx), gmix(c.y, d.y, fx), fy);
    return gmix(gmix(a.w, b.w, fx), gmix(c.w, d.w, fx), fy);
}

__device__ __forceinline__ float2 sed_bilinear(const Scene& S, float px, float py) {
    const float2 z = make_float2(0.0f, 0.0f);
    if (!(px > -2.0f && px < (float)S.n + 1.0f && py > -2.0f && py < (float)S.n + 1.0f)) return z;
    const int ix = (int)px, iy = (int)py;
    const float fx = fract_(px), fy = fract_(py);
    auto t = [&](int x, int y) {
        return (x >= 0 && x < S.n && y >= 0 && y < S.n) ? __ldg(S.sed + (size_t)y * S.n + x) : z;
    };
    const float2 a = t(ix, iy), b = t(ix + 1, iy), c = t(ix, iy + 1), d = t(ix + 1, iy + 1);
    return make_float2(gmix(gmix(a.x, b.x, fx), gmix(c.x, d.x, fx), fy),
                       gmix(gmix(a.y, b.y, fx), gmix(c.y, d.y, fx), fy));
}

struct Ray {
    V3 pos;
    float w;  // penumbra (min sdf) or 0
    float dist;
    float4 terr;
};

// raymarch (glsl/rendering.glsl:462-516)
__device__ __noinline__ Ray raymarch(const Scene S, V3 o, V3 d, float max_d, int max_iter, int kind) {
    float dist = 0.001f, d_dist = 0.1f;
    const bool terrain = kind == KIND_TERRAIN;
    if (terrain) {
        dist = 0.0f;
        d_dist = 0.1e-12f;
    }
    float min_sdf = 1.0f;
    // each step needs only the marched height; the full texel (terr) is
    // sampled again where the ray stops
    V3 last = o;
    bool sampled = false;
    for (int i = 0; i < max_iter; ++i) {
        const V3 sp = add(o, scl(d, dist));
        const float t_height = tex_height(S, sp.x, sp.z, terrain);
        last = sp;
        sampled = true;
        if ((sp.y > S.max_height && d.y >= 0.0f) || (sp.y <= 0.0f && d.y < 0.0f)) break;
        const float d_height = sp.y - t_height;
        if (fabsf(d_height) <= 0.05f) {
            const V3 q = sub(sp, scl(d, 0.05f));
            return Ray{q, 0.0f, dist - 0.05f, tex_bilinear(S, q.x, q.z)};
        } else if (d_height < 0.0f) {
            return Ray{add(o, scl(d, dist)), min_sdf, dist, tex_bilinear(S, sp.x, sp.z)};
        }
        min_sdf = gmin(min_sdf, 12.0f * d_dist / dist);
        if (dist > max_d) return Ray{sp, min_sdf, max_d, tex_bilinear(S, sp.x, sp.z)};
        d_dist = S.prec * d_height;
        dist += d_dist;
    }
    const float4 terr = sampled ? tex_bilinear(S, last.x, last.z) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    return Ray{add(o, scl(d, max_d)), min_sdf, max_d, terr};
}

__device__ __forceinline__ float fog_mix(float f) { return gclamp(f * f, 0.0f, 1.0f); }

// get_material_color (glsl/rendering.glsl:115-146)
__device__ V3 material_color(const Ray& ray, V3 norm, const Materials& m) {
    const float cos_a = dot(norm, v3(-0.0f, -1.0f, -0.0f));
    const float dirt = smoothstep(0.0f, 1.0f, gmin(1.0f, ray.terr.y));
    V3 col = m.rock;
    if (dirt > 0.0f) {
        if (cos_a < 0.75f) {
            const float wet = 1.0f - smoothstep(0.25f, 0.75f, cos_a);
            col = mix3(m.dirt, scl(m.dirt, 0.4f), wet);
        } else if (cos_a < 0.95f) {
            const float dc = 1.0f - smoothstep(0.85f, 0.95f, cos_a);
            col = mix3(m.grass, m.dirt, dc);
        } else {
            col = m.grass;
        }
        col = mix3(m.rock, col, dirt);
    } else {
        const float steep = 1.0f - smoothstep(0.0f, 0.65f, cos_a);
        col = mix3(m.rock, scl(m.rock, 0.5f), steep);
    }
    return col;
}

__device__ __forceinline__ Materials ambient_materials() {
    return Materials{v3(0.00014f, 0.00084f, 0.00018f), v3(0.0008f, 0.0008f, 0.0008f), v3(0.00032f, 0.00030f, 0.0018f)};
}
__device__ __forceinline__ Materials diffuse_materials() {
    return Materials{v3(0.2068f * 1.3f / 5.0f, 0.279f * 1.3f / 5.0f, 0.01f * 1.3f / 5.0f),
                     v3(0.40f * 1.3f / 6.0f, 0.39f * 1.3f / 6.0f, 0.37f * 1.3f / 6.0f),
                     v3(0.1968f * 1.3f / 6.0f, 0.169f * 1.3f / 6.0f, 0.03f * 1.3f / 6.0f)};
}

__device__ __forceinline__ V3 sky_base() { return v3(0.3f, 0.5f, 0.85f); }

// get_img_normal (:160-172): terrain normal from rock + dirt
__device__ V3 terrain_normal(const Scene& S, float x, float z) {
    const float4 r = tex_bilinear(S, x + 1.0f, z + 0.0f), l = tex_bilinear(S, x + -1.0f, z + 0.0f);
    const float4 b = tex_bilinear(S, x + 0.0f, z + -1.0f), t = tex_bilinear(S, x + 0.0f, z + 1.0f);
    const float dx = r.x + r.y - l.x - l.y;
    const float dz = t.x + t.y - b.x - b.y;
    return normalize(cross(v3(2.0f, dx, 0.0f), v3(0.0f, dz, 2.0f)));
}

// get_img_normal_w (:148-157): water surface normal from the total height
__device__ V3 water_normal(const Scene& S, float x, float z) {
    const float dx = tex_bilinear(S, x + 1.0f, z + 0.0f).w - tex_bilinear(S, x + -1.0f, z + 0.0f).w;
    const float dz = tex_bilinear(S, x + 0.0f, z + 1.0f).w - tex_bilinear(S, x + 0.0f, z + -1.0f).w;
    return normalize(cross(v3(2.0f, dx, 0.0f), v3(0.0f, dz, 2.0f)));
}

// get_fog_color (:174-180)
__device__ V3 fog_color(V3 col, float ray_dist, float sundot) {
    const float fo = 1.0f - rm_exp(-rm_pow(0.15f * ray_dist / MAX_DIST, 2.5f));
    const float p = rm_pow(sundot * 1.5f, 4.0f);
    const V3 fco = add(scl(v3(0.4f, 0.65f, 1.0f), 0.65f), scl(scl(v3(1.0f, 0.8f, 0.5f), 0.1f), p));
    return mix3(col, fco, fo);
}

// get_sky_color (:182-220)
__device__ V3 sky_color(V3 dir, float sundot) {
    const float diry = dir.y;
    const float dd = diry * diry * 0.37f;
    const V3 s = sky_base();
    V3 col = v3(s.x - dd, s.y - dd, s.z - dd);
    col = mix3(col, scl(v3(0.7f, 0.75f, 0.85f), 0.85f), rm_pow(1.0f - gmax(diry, 0.0f), 4.0f));
    col = add(col, scl(scl(v3(1.0f, 0.7f, 0.4f), 0.25f), rm_pow(sundot, 5.0f)));
    col = add(col, scl(scl(v3(1.0f, 0.8f, 0.6f), 0.25f), rm_pow(sundot, 64.0f)));
    col = add(col, scl(scl(v3(1.0f, 0.8f, 0.6f), 0.2f), rm_pow(sundot, 512.0f)));
    return mix3(col, scl(v3(0.4f, 0.65f, 1.0f), 0.68f), rm_pow(1.0f - gmax(diry, 0.0f), 16.0f));
}

struct Shade {
    V3 rgb;
    float w;
};

// get_shade (:227-283)
__device__ __noinline__ Shade shade(const Scene S, const Ray ray, V3 normal, bool is_water) {
    const float shadow_diff = S.max_height - ray.pos.y;
    const float shadow_scale = shadow_diff / -S.light.y;
    const float shadow_max = len(scl(S.light, shadow_scale));
    const Ray shadow = raymarch(S, ray.pos, neg(S.light), shadow_max, MAX_STEPS / 2, KIND_TERRAIN);
    const float amb_factor = gclamp(0.5f + 0.5f * -normal.y, 0.0f, 1.0f);
    V3 ambient, diffuse;
    if (is_water) {
        ambient = scl(sky_base(), 0.005f);
        diffuse = scl(v3(0.108f, 0.187f, 0.288f), 0.1f);
    } else {
        ambient = material_color(ray, neg(normal), ambient_materials());
        diffuse = material_color(ray, normal, diffuse_materials());
    }
    ambient = add(ambient, scl(add(diffuse, scl(sky_base(), 0.01f)), amb_factor * 0.20f));
    Shade out{ambient, 0.04f};
    if (shadow.dist >= shadow_max) {
        const float lambrt = gmax(dot(S.light, normal), 0.0f);
        out.rgb = add(out.rgb, scl(scl(diffuse, lambrt), shadow.w));
        out.w = shadow.w;
    }
    return out;
}

// get_terrain_color (:289-302)
__device__ V3 terrain_color(const Scene& S, const Ray& ray, V3 dir, float sundot) {
    const V3 normal = terrain_normal(S, ray.pos.x, ray.pos.z);
    V3 col = shade(S, ray, normal, false).rgb;
    col = fog_color(col, ray.dist, sundot);
    return mix3(col, sky_color(dir, sundot), fog_mix(ray.dist / MAX_DIST));
}

// refractCameraRay (:304-317)
__device__ V3 refract_ray(V3 n, V3 d, float eta) {
    const float cos_t = dot(neg(n), d);
    const float sin_t2 = 1.0f - cos_t * cos_t;
    const float sin_p2 = eta * eta * sin_t2;
    if (sin_p2 > 1.0f) return reflect(d, n);
    const float cos_p = sqrtf(1.0f - sin_p2);
    return add(scl(d, eta), scl(n, eta * cos_t - cos_p));
}

// get_water_color (:319-391)
__device__ V3 water_color(const Scene& S, const Ray& w_ray, V3 dir, float sundot) {
    const V3 w_norm = water_normal(S, w_ray.pos.x, w_ray.pos.z);
    const V3 refract_dir = refract_ray(w_norm, dir, 1.0f / 1.3f);
    Ray t_ray = raymarch(S, w_ray.pos, neg(refract_dir), MAX_DIST / 8.0f, MAX_STEPS / 4, KIND_TERRAIN);
    const float water_vol = t_ray.dist;
    t_ray.dist += w_ray.dist;
    const V3 t_shad = terrain_color(S, t_ray, dir, sundot);
    const V3 w_refl = reflect(dir, w_norm);
    Ray wrefl_ray = raymarch(S, w_ray.pos, w_refl, MAX_DIST, MAX_STEPS, KIND_TERRAIN);
    const Shade w_shad = shade(S, w_ray, w_norm, true);
    V3 water_col = w_shad.rgb;
    const float refl_sundot = gclamp(dot(w_refl, neg(S.light)), 0.0f, 1.0f);
    const V3 wrefl_skycol = sky_color(w_refl, refl_sundot);
    const float cos_theta = dot(dir, w_norm);
    const float fresnel = gmax(rm_pow(1.0f - cos_theta, 2.0f), 0.06f);
    if (wrefl_ray.dist >= MAX_DIST) {
        water_col = mix3(t_shad, water_col, gmin(1.0f, water_vol / 2.0f));
        water_col = mix3(water_col, wrefl_skycol, fresnel);
        water_col = mix3(w_shad.rgb, water_col, w_shad.w);
    } else {
        wrefl_ray.dist += w_ray.dist;
        water_col = mix3(t_shad, water_col, gmin(1.0f, water_vol / 2.0f));
        water_col = mix3(water_col, terrain_color(S, wrefl_ray, w_refl, refl_sundot), w_shad.w);
        water_col = mix3(t_shad, water_col, fresnel);
        water_col = mix3(water_col, wrefl_skycol, fog_mix(wrefl_ray.dist / MAX_DIST));
    }
    return water_col;
}

struct RenderArgs {
    Scene S;
    float inv_p[16];  // inverse(perspective), column-major
    float inv_v[16];  // inverse(view)
    V3 pos;
    int draw_water;
    int display_sediment;
    float sediment_max_cap;
    int low_res;
    int wd, hd;   // dispatch size (pixels marched)
    int width;    // output row length
    float alpha;  // stored alpha (0, or clamp(hmap_dims.x) in the low-resolution form)
    uchar4* rgba;
    float* rgb;   // optional float colour (after gamma)
};

// to_world (:518-523): inverse(perspective) * c, / w, inverse(view) * c
__device__ __forceinline__ float4 mat_vec(const float* m, float4 v) {
    float4 r;
    r.x = m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w;
    r.y = m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w;
    r.z = m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w;
    r.w = m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w;
    return r;
}
__device__ __forceinline__ float4 to_world(const RenderArgs& a, float4 c) {
    c = mat_vec(a.inv_p, c);
    const float w = c.w;
    c = make_float4(c.x / w, c.y / w, c.z / w, c.w / w);
    return mat_vec(a.inv_v, c);
}

__device__ __forceinline__ unsigned char unorm8(float f) {
    f = f > 0.0f ? (f < 1.0f ? f : 1.0f) : 0.0f;  // NaN -> 0
    return (unsigned char)floorf(f * 255.0f + 0.5f);
}

// main (:525-539) and get_pixel_color (:393-460).  Eight blocks per SM (a
// 64-register cap with small spills) hide the marches' latencies better
// than five unspilled ones (9 % faster).
__global__ void __launch_bounds__(128, 8) k_render(const RenderArgs a) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= a.wd || py >= a.hd) return;
    const Scene S = a.S;
    const float ux = (float)px / (float)a.wd, uy = (float)py / (float)a.hd;
    const float cx = 2.0f * ux - 1.0f, cy = 2.0f * uy - 1.0f;
    const float4 rs = to_world(a, make_float4(0.0f, 0.0f, -1.0f, 1.0f));
    const float4 re = to_world(a, make_float4(cx, cy, 1.0f, 1.0f));
    const V3 dir = normalize(v3(re.x - rs.x, re.y - rs.y, re.z - rs.z));

    const Ray ray = raymarch(S, a.pos, dir, MAX_DIST, MAX_STEPS, KIND_TOTAL);
    const float sundot = gclamp(dot(dir, neg(S.light)), 0.0f, 1.0f);
    const float pxz = ray.pos.x * 1.0f, pzz = ray.pos.z * 1.0f;
    const float water_h = gmin(1.0f, smoothstep(1e-4f, 1.0f, ray.terr.z));
    V3 color;
    if (pxz < 0.0f || pxz >= (float)S.n || pzz < 0.0f || pzz >= (float)S.n) {
        color = sky_color(dir, sundot);
    } else if (ray.dist >= MAX_DIST) {
        color = sky_color(dir, sundot);
    } else if (water_h > 1e-12f && a.draw_water) {
        V3 wc = water_color(S, ray, dir, sundot);
        wc = fog_color(wc, ray.dist, sundot);
        color = mix3(wc, sky_color(dir, sundot), fog_mix(ray.dist / MAX_DIST));
    } else {
        color = terrain_color(S, ray, dir, sundot);
    }
    if (a.display_sediment) {
        const float2 sd = sed_bilinear(S, ray.pos.x, ray.pos.z);
        const float r = gmin(1.0f, sd.x / a.sediment_max_cap);
        const float g = gmin(1.0f, sd.y / a.sediment_max_cap);
        color = mix3(color, v3(1.0f, 0.0f, 0.0f), r);
        color = mix3(color, v3(0.0f, 1.0f, 0.0f), g);
    }
    const float gam = 1.0f / 2.2f;
    color = v3(rm_pow(color.x, gam), rm_pow(color.y, gam), rm_pow(color.z, gam));
    const uchar4 q = make_uchar4(unorm8(color.x), unorm8(color.y), unorm8(color.z), unorm8(a.alpha));
    const int rep = a.low_res ? 3 : 1;
    for (int oy = 0; oy < rep; ++oy)
        for (int ox = 0; ox < rep; ++ox) {
            const size_t o = (size_t)(py * rep + oy) * a.width + (px * rep + ox);
            a.rgba[o] = q;
            if (a.rgb) {
                a.rgb[3 * o + 0] = color.x;
                a.rgb[3 * o + 1] = color.y;
                a.rgb[3 * o + 2] = color.z;
            }
        }
}

__global__ void k_pack_heightmap(const float* __restrict__ rock, const float* __restrict__ dirt,
                                 const float* __restrict__ water, const float* __restrict__ s0,
                                 const float* __restrict__ s1, size_t count, float4* __restrict__ hm,
                                 float2* __restrict__ sed) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        const float r = rock[i], g = dirt ? dirt[i] : 0.0f, b = water[i];
        hm[i] = make_float4(r, g, b, r + g + b);
        if (sed) sed[i] = make_float2(s0[i], s1 ? s1[i] : 0.0f);
    }
}

// Gauss-Jordan inverse with partial pivoting in double, rounded to float;
// false for a singular matrix
bool invert4(const float* m, float* out) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            a[r][c] = m[c * 4 + r];
            a[r][4 + c] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[p][c])) p = r;
        if (a[p][c] == 0.0 || !std::isfinite(a[p][c])) return false;
        if (p != c)
            for (int k = 0; k < 8; ++k) std::swap(a[p][k], a[c][k]);
        const double inv = 1.0 / a[c][c];
        for (int k = 0; k < 8; ++k) a[c][k] *= inv;
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            const double f = a[r][c];
            if (f == 0.0) continue;
            for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[c * 4 + r] = (float)a[r][4 + c];
    return true;
}

}  // namespace

int render_image(const RenderInput& in, const hg_camera& cam, int width, int height, uint8_t* rgba_dev,
                 float* rgb_dev, cudaStream_t st) {
    RenderArgs a{};
    if (!invert4(cam.perspective, a.inv_p) || !invert4(cam.view, a.inv_v)) return HG_ERR_INVALID;
    const size_t cells = (size_t)in.n * in.n;
    const int blocks = (int)std::min<size_t>((cells + 255) / 256, 152 * 16);
    k_pack_heightmap<<<blocks, 256, 0, st>>>(in.rock, in.dirt, in.water, in.sed0, in.sed1, cells, in.hm,
                                             cam.display_sediment ? in.sed : nullptr);
    count_launch();
    // the light direction, normalize(vec3(0, -0.7, 1)), in float as the kernel would
    const float lx = 0.0f, ly = -0.7f, lz = 1.0f;
    const float ll = std::sqrt(lx * lx + ly * ly + lz * lz);
    a.S = Scene{in.hm, in.sed, in.n, in.max_height, cam.prec, V3{lx / ll, ly / ll, lz / ll}};
    a.pos = V3{cam.pos[0], cam.pos[1], cam.pos[2]};
    a.draw_water = cam.draw_water;
    a.display_sediment = cam.display_sediment;
    a.sediment_max_cap = cam.sediment_max_cap;
    a.low_res = cam.low_res_div3 ? 1 : 0;
    a.wd = a.low_res ? width / 3 : width;
    a.hd = a.low_res ? height / 3 : height;
    a.width = width;
    a.alpha = a.low_res ? (float)in.hmap_dim_x : 0.0f;
    a.rgba = reinterpret_cast<uchar4*>(rgba_dev);
    a.rgb = rgb_dev;
    if (a.low_res) {
        cudaMemsetAsync(rgba_dev, 0, (size_t)width * height * 4, st);
        if (rgb_dev) cudaMemsetAsync(rgb_dev, 0, (size_t)width * height * 3 * sizeof(float), st);
    }
    if (a.wd > 0 && a.hd > 0) {
        dim3 blk(16, 8), grid((a.wd + 15) / 16, (a.hd + 7) / 8);
        k_render<<<grid, blk, 0, st>>>(a);
        count_launch();
    }
    return HG_OK;
}

}  // namespace hg
