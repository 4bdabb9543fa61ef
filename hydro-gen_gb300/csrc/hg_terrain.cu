// hydro-gen's own terrain generator and rain, on the GPU.
//
//   hg_init_reference_heightmap   glsl/heightmap.glsl:52-158 (masks :25-43),
//                                 via World::gen_heightmap (src/state.cpp:116-147)
//   HG_RAIN_REFERENCE             glsl/rain.glsl:32-56 (cadence src/main.cpp:315-319)
//
// Noise (the shaders take these from glNoise, glsl/simplex_noise.glsl):
//   simplex2   2-D simplex noise as published by McEwan, Sheets, Gustavson and
//              Richardson ("Efficient computational noise in GLSL", JGT 2012):
//              skewed lattice, permutation polynomial (34 x^2 + x) mod 289,
//              gradients from 41 points on a line folded onto a diamond
//   gnoise_d   gradient noise with quintic fade and analytic derivatives
//              (Inigo Quilez's formulation), corner gradients from Hugo
//              Elias's integer hash (wrap-around int32 arithmetic)
//   fbm_*      octave sums; the "erosion" variant divides each octave by
//              1 + |running sum of derivatives|^2
// Float arithmetic in the shaders' operation order (the library is built
// without contraction), so the CPU restatement reproduces every bit except
// where exp() enters (the exponential mask).  pow(x, 2) and pow(x, 3) of
// possibly negative bases are x*x and x*x*x (GLSL leaves pow undefined for
// x < 0) and pow(r, 1) is r.
#include <cmath>

#include "hg_internal.h"

namespace hg {

namespace {

constexpr int BX = 32, BY = 8;

struct Fbm {  // gln_tFBMOpts with redistribution 1 (what every call site passes)
    float seed, persistance, lacunarity, scale;
    int octaves;
    bool turbulence, ridge;
};

__device__ __forceinline__ float fract_(float x) { return x - floorf(x); }
__device__ __forceinline__ float mod289(float x) { return x - 289.0f * floorf(x / 289.0f); }
__device__ __forceinline__ float perm(float x) { return mod289((x * 34.0f + 1.0f) * x); }

__device__ float simplex2(float vx, float vy) {
    const float F = 0.366025403784439f;   // (sqrt(3) - 1) / 2
    const float G = 0.211324865405187f;   // (3 - sqrt(3)) / 6
    const float G2 = -0.577350269189626f; // 2 G - 1
    const float R = 0.024390243902439f;   // 1 / 41
    const float s = vx * F + vy * F;
    float ix = floorf(vx + s), iy = floorf(vy + s);
    const float t = ix * G + iy * G;
    const float x0 = vx - ix + t, y0 = vy - iy + t;
    const float ox = x0 > y0 ? 1.0f : 0.0f, oy = x0 > y0 ? 0.0f : 1.0f;
    const float cx[3] = {x0, x0 + G - ox, x0 + G2};
    const float cy[3] = {y0, y0 + G - oy, y0 + G2};
    ix = mod289(ix);
    iy = mod289(iy);
    const float row[3] = {perm(iy + 0.0f), perm(iy + oy), perm(iy + 1.0f)};
    const float col[3] = {0.0f, ox, 1.0f};
    float sum = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float h = perm(row[k] + ix + col[k]);
        float w = gmax(0.5f - (cx[k] * cx[k] + cy[k] * cy[k]), 0.0f);
        w = w * w;
        w = w * w;
        const float gx = 2.0f * fract_(h * R) - 1.0f;
        const float gy = fabsf(gx) - 0.5f;
        const float a = gx - floorf(gx + 0.5f);
        w *= 1.79284291400159f - 0.85373472095314f * (a * a + gy * gy);
        const float d = a * cx[k] + gy * cy[k];
        sum = k == 0 ? w * d : sum + w * d;
    }
    return 130.0f * sum;
}

__device__ __forceinline__ void elias_gradient(int32_t px, int32_t py, float& gx, float& gy) {
    uint32_t n[2] = {(uint32_t)px * 3u + (uint32_t)py * 311u, (uint32_t)px * 37u + (uint32_t)py * 113u};
    float g[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        uint32_t v = (n[k] << 13) ^ n[k];
        v = v * (v * v * 15731u + 789221u) + 1376312589u;
        g[k] = -1.0f + 2.0f * (float)(int32_t)(v & 0x0fffffffu) / 268435455.0f;
    }
    gx = g[0];
    gy = g[1];
}

// value (n) and gradient (dx, dy) of the gradient noise at (px, py)
__device__ void gnoise_d(float px, float py, float& nv, float& ddx, float& ddy) {
    const float flx = floorf(px), fly = floorf(py);
    const int32_t ix = (int32_t)flx, iy = (int32_t)fly;
    const float fx = px - flx, fy = py - fly;
    const float ux = fx * fx * fx * (fx * (fx * 6.0f - 15.0f) + 10.0f);
    const float uy = fy * fy * fy * (fy * (fy * 6.0f - 15.0f) + 10.0f);
    const float dux = 30.0f * fx * fx * (fx * (fx - 2.0f) + 1.0f);
    const float duy = 30.0f * fy * fy * (fy * (fy - 2.0f) + 1.0f);
    float ax, ay, bx, by, cx, cy, ex, ey;  // corners (0,0), (1,0), (0,1), (1,1)
    elias_gradient(ix, iy, ax, ay);
    elias_gradient(ix + 1, iy, bx, by);
    elias_gradient(ix, iy + 1, cx, cy);
    elias_gradient(ix + 1, iy + 1, ex, ey);
    const float va = ax * (fx - 0.0f) + ay * (fy - 0.0f);
    const float vb = bx * (fx - 1.0f) + by * (fy - 0.0f);
    const float vc = cx * (fx - 0.0f) + cy * (fy - 1.0f);
    const float vd = ex * (fx - 1.0f) + ey * (fy - 1.0f);
    const float k = va - vb - vc + vd;
    const float uu = ux * uy;
    nv = va + ux * (vb - va) + uy * (vc - va) + uu * k;
    ddx = ax + ux * (bx - ax) + uy * (cx - ax) + uu * (ax - bx - cx + ex) + dux * (uy * k + vb - va);
    ddy = ay + ux * (by - ay) + uy * (cy - ay) + uu * (ay - by - cy + ey) + duy * (ux * k + vc - va);
}

__device__ float fbm_simplex(float vx, float vy, const Fbm& o) {
    vx += o.seed * 100.0f;
    vy += o.seed * 100.0f;
    float acc = 0.0f, amp = 1.0f, freq = 1.0f, norm = amp;
    for (int i = 0; i < o.octaves && i < 30; ++i) {  // MAX_FBM_ITERATIONS
        float v = simplex2(vx * freq * o.scale, vy * freq * o.scale);
        if (o.turbulence) v = fabsf(v);
        if (o.turbulence && o.ridge) v = 1.0f - v;
        acc += v * amp;
        freq *= o.lacunarity;
        amp *= o.persistance;
        norm += amp;
    }
    return acc / norm;
}

__device__ float fbm_gradient(float vx, float vy, const Fbm& o) {
    vx += o.seed * 100.0f;
    vy += o.seed * 100.0f;
    float acc = 0.0f, amp = 1.0f, freq = 1.0f, norm = amp;
    for (int i = 0; i < o.octaves && i < 30; ++i) {  // MAX_FBM_ITERATIONS
        float nv, dx, dy;
        gnoise_d(vx * freq * o.scale, vy * freq * o.scale, nv, dx, dy);
        float v = (nv + 1.0f) / 2.0f;
        if (o.turbulence) v = fabsf(v);
        if (o.turbulence && o.ridge) v = 1.0f - v;
        acc += v * amp;
        freq *= o.lacunarity;
        amp *= o.persistance;
        norm += amp;
    }
    return acc / norm;
}

// erosion-like fBm: octaves damped by the running sum of derivatives
__device__ float fbm_eroded(float vx, float vy, const Fbm& o) {
    vx += o.seed * 100.0f;
    vy += o.seed * 100.0f;
    float acc = 0.0f, amp = 1.0f, freq = 1.5f, norm = amp, sx = 0.0f, sy = 0.0f;
    for (int i = 0; i < o.octaves && i < 30; ++i) {  // MAX_FBM_ITERATIONS
        float nv, dx, dy;
        gnoise_d(vx * freq * o.scale, vy * freq * o.scale, nv, dx, dy);
        if (o.turbulence) { nv = fabsf(nv); dx = fabsf(dx); dy = fabsf(dy); }
        if (o.turbulence && o.ridge) { nv = 1.0f - nv; dx = 1.0f - dx; dy = 1.0f - dy; }
        sx += dx;
        sy += dy;
        const float v = (nv + 1.0f) / 2.0f;
        acc += v * amp / (1.0f + (sx * sx + sy * sy));
        freq *= o.lacunarity;
        amp *= o.persistance;
        norm += amp;
    }
    return acc / norm;
}

__global__ void k_ref_heightmap(const hg_map_settings cfg, int n, float* __restrict__ rock, float* __restrict__ dirt) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= n || y >= n) return;
    const float fx = (float)x, fy = (float)y;
    const float uvx = fx / (float)n, uvy = fy / (float)n;
    const Fbm opts{cfg.seed, cfg.persistance, cfg.lacunarity, cfg.scale, cfg.octaves, false, false};
    const float ws = cfg.domain_warp_scale;
    // domain warp (:65-77)
    float wx = 1.0f, wy = 1.0f;
    if (cfg.domain_warp != 0) {
        wx = fbm_gradient(fx + 2.3f, fy + 2.9f, opts);
        wy = fbm_gradient(fx - 3.1f, fy - 4.3f, opts);
        if (cfg.domain_warp == 2) {
            const float ax = fbm_gradient(fx + ws * wx - 5.7f, fy + ws * wy + 27.9f, opts);
            const float ay = fbm_gradient(fx + ws * wx + 11.5f, fy + ws * wy - 23.7f, opts);
            wx = ax;
            wy = ay;
        }
    }
    float val = fbm_eroded(fx + ws * wx, fy + ws * wy, opts);  // :78-83
    float hm = cfg.height_mult;
    if (cfg.uplift != 0) {  // :85-101
        const Fbm up_opts{cfg.seed, cfg.persistance, cfg.lacunarity, cfg.scale / cfg.uplift_scale, cfg.octaves,
                          true, true};
        const float up = fbm_simplex(fx - 7.3f, fy + 19.9f, up_opts);
        if (cfg.mask_exp != 0) hm += 2.5f;
        hm += 1.0f;
        val *= up;
    }
    if (cfg.mask_round != 0) {  // :102-107, round_mask :25-29
        if (cfg.mask_exp != 0) hm += 16.0f;
        const float ax = uvx - 0.5f, ay = uvy - 0.5f;
        const float v = 1.0f - (ax * ax + ay * ay + 0.75f);
        val = val * gmax(0.0f, v * 1.0f);
    }
    if (cfg.mask_exp != 0) {  // :108-111, exp_mask :42-44
        hm += 2.0f;
        val = val * (expf(val) - 1.0f) / 1.718f;
    }
    if (cfg.mask_power != 0) {  // :112-118, power_mask :38-40
        hm += 1.25f;
        if (cfg.mask_exp != 0) hm += 2.0f;
        const float b = val + 0.5f;
        val = val * (((b * b * b - 0.125f) / 3.25f) * 0.55f + 0.45f);
    }
    if (cfg.mask_slope != 0) val = 0.25f * val + 0.75f * (val * uvx * uvy);  // slope_mask :34-36
    val = val + (float)(4u * cfg.mask_round) * val;
    if (cfg.terrace > 0) {  // :124-129
        const float q = 1.0f / ((float)cfg.terrace * hm);
        const float lvl = floorf(val / q);
        const float t = cfg.terrace_scale;
        val = (t * lvl * q) + val * (1.0f - t);
    }
    const size_t i = (size_t)y * n + x;
    rock[i] = gmin(cfg.max_height, val * cfg.max_height * hm);  // :131
    if (dirt) dirt[i] = (fbm_gradient(fx + 13.7f, fy + 27.1f, opts) + 1.5f) * cfg.max_dirt;  // :133-135
}

struct RefRain {
    float seed, amount, mountain_thresh, mountain_multip, drops, max_height;
};

// water += amount r + mountain bonus, r = max(0, simplex fBm); total height
// (rock + dirt) + water
__global__ void k_ref_rain(const RefRain rr, int n, const float* __restrict__ rock, const float* __restrict__ dirt,
                           float* __restrict__ water) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= n || y >= n) return;
    const size_t i = (size_t)y * n + x;
    const Fbm opts{rr.seed, 0.5f, 2.0f, rr.drops, 8, false, false};
    const float r = gmax(0.0f, fbm_simplex((float)x, (float)y, opts));
    float incr = rr.amount * r;
    const float total = (dirt ? rock[i] + dirt[i] : rock[i] + 0.0f) + water[i];
    const float mountain = total - rr.max_height * rr.mountain_thresh;
    if (mountain > 0.0f)
        incr += mountain * rr.mountain_multip * r / ((1.0f - rr.mountain_thresh) * rr.max_height);
    water[i] = water[i] + incr;
}

dim3 grid_for(int n) { return dim3((n + BX - 1) / BX, (n + BY - 1) / BY); }

}  // namespace

void launch_ref_heightmap(const hg_map_settings& cfg, int n, float* rock, float* dirt, cudaStream_t st) {
    k_ref_heightmap<<<grid_for(n), dim3(BX, BY), 0, st>>>(cfg, n, rock, dirt);
    count_launch();
}

void launch_ref_rain(const hg_rain_settings& rs, const hg_map_settings& map, float time, int n, const float* rock,
                     const float* dirt, float* water, cudaStream_t st) {
    RefRain rr;
    volatile float tf = time * 1.372914227e3f;  // glsl/rain.glsl:36: fract(time * 1.372914227e3) * 1000
    rr.seed = ((float)tf - std::floor((float)tf)) * 1000.0f;
    rr.amount = rs.amount;
    rr.mountain_thresh = rs.mountain_thresh;
    rr.mountain_multip = rs.mountain_multip;
    rr.drops = rs.drops;
    rr.max_height = map.max_height;
    k_ref_rain<<<grid_for(n), dim3(BX, BY), 0, st>>>(rr, n, rock, dirt, water);
    count_launch();
}

}  // namespace hg
