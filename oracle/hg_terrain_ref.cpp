// CPU restatement of hydro-gen's own terrain generator and rain — TEST
// INFRASTRUCTURE ONLY (checks hg_terrain.cu).  Float arithmetic in the
// shaders' operation order (built without contraction), so the GPU kernels
// match bit for bit except where exp() enters (the exponential mask).
//
//   heightmap generator   glsl/heightmap.glsl:25-158 (masks :25-43, main :52-158)
//   noise                 glsl/simplex_noise.glsl: gln_simplex :377-402,
//                         gln_sfbm :419-456, hash :575-583, noised :586-607,
//                         perlfbm :609-646, erosion_perlfbm :648-688
//   rain                  glsl/rain.glsl:32-56
//
// The simplex noise is the published 2-D algorithm of McEwan, Sheets,
// Gustavson and Richardson ("Efficient computational noise in GLSL", JGT
// 2012: skewed lattice, mod-289 permutation polynomial, gradients from a
// ring of 41 points); the gradient noise with analytic derivatives is Inigo
// Quilez's (gradient noise with quintic fade and its derivatives), its corner
// gradients from Hugo Elias's integer hash; the fBm with derivative damping
// divides each octave by 1 + |sum of derivatives|^2.  The shaders vendor these
// from glNoise (no version pinned) and evaluate them in float.
//
// Two shader expressions have no defined float meaning and are read as
// intended: pow(x, 2.0) and pow(x, 3) of possibly negative bases are x*x and
// x*x*x (GLSL leaves pow undefined for x < 0), and pow(result, 1.0) is result.
#include <cmath>
#include <cstdint>

namespace {

struct MapSettings {  // Map_settings_data, glsl/bindings.glsl:70-99 (std140, 96 B)
    float max_height, max_dirt;
    int32_t hmap_dims[2];
    float height_mult, water_lvl, seed, persistance, lacunarity, scale, redistribution;
    int32_t octaves;
    uint32_t fake_erosion, mask_round, mask_exp, mask_power, mask_slope, uplift;
    float uplift_scale;
    int32_t domain_warp;
    float domain_warp_scale;
    int32_t terrace;
    float terrace_scale;
    float pad;
};
static_assert(sizeof(MapSettings) == 96, "std140 size");

struct FbmOpts {  // gln_tFBMOpts
    float seed, persistance, lacunarity, scale, redistribution;
    int octaves;
    bool turbulence, ridge;
};

float gfract(float x) { return x - std::floor(x); }
float gmod(float x, float y) { return x - y * std::floor(x / y); }
float perm289(float x) { return gmod((x * 34.0f + 1.0f) * x, 289.0f); }
float gmaxf(float x, float y) { return x < y ? y : x; }
float gminf(float x, float y) { return y < x ? y : x; }

float simplex(float vx, float vy) {
    const float Cx = 0.211324865405187f, Cy = 0.366025403784439f, Cz = -0.577350269189626f,
                Cw = 0.024390243902439f;
    float s = vx * Cy + vy * Cy;
    float ix = std::floor(vx + s), iy = std::floor(vy + s);
    float t = ix * Cx + iy * Cx;
    float x0 = vx - ix + t, y0 = vy - iy + t;
    float i1x = x0 > y0 ? 1.0f : 0.0f, i1y = x0 > y0 ? 0.0f : 1.0f;
    float x1 = x0 + Cx - i1x, y1 = y0 + Cx - i1y;
    float x2 = x0 + Cz, y2 = y0 + Cz;
    ix = gmod(ix, 289.0f);
    iy = gmod(iy, 289.0f);
    float q0 = perm289(iy + 0.0f), q1 = perm289(iy + i1y), q2 = perm289(iy + 1.0f);
    float p[3] = {perm289(q0 + ix + 0.0f), perm289(q1 + ix + i1x), perm289(q2 + ix + 1.0f)};
    float m[3] = {gmaxf(0.5f - (x0 * x0 + y0 * y0), 0.0f), gmaxf(0.5f - (x1 * x1 + y1 * y1), 0.0f),
                  gmaxf(0.5f - (x2 * x2 + y2 * y2), 0.0f)};
    const float gx_[3] = {x0, x1, x2}, gy_[3] = {y0, y1, y2};
    float dot = 0.0f;
    for (int k = 0; k < 3; ++k) {
        m[k] = m[k] * m[k];
        m[k] = m[k] * m[k];
        float xx = 2.0f * gfract(p[k] * Cw) - 1.0f;
        float h = std::fabs(xx) - 0.5f;
        float ox = std::floor(xx + 0.5f);
        float a0 = xx - ox;
        m[k] *= 1.79284291400159f - 0.85373472095314f * (a0 * a0 + h * h);
        float g = a0 * gx_[k] + h * gy_[k];
        dot = k == 0 ? m[k] * g : dot + m[k] * g;
    }
    return 130.0f * dot;
}

float redistribute(float r, float e) { return e == 1.0f ? r : std::pow(r, e); }

float sfbm(float vx, float vy, const FbmOpts& o) {
    vx += o.seed * 100.0f;
    vy += o.seed * 100.0f;
    float result = 0.0f, amp = 1.0f, freq = 1.0f, maximum = amp;
    for (int i = 0; i < o.octaves && i < 30; ++i) {  // MAX_FBM_ITERATIONS
        float v = simplex(vx * freq * o.scale, vy * freq * o.scale);
        if (o.turbulence) v = std::fabs(v);
        if (o.turbulence && o.ridge) v = 1.0f - v;
        result += v * amp;
        freq *= o.lacunarity;
        amp *= o.persistance;
        maximum += amp;
    }
    return redistribute(result, o.redistribution) / maximum;
}

void hash2(int32_t px, int32_t py, float& gx, float& gy) {
    uint32_t n[2] = {(uint32_t)px * 3u + (uint32_t)py * 311u, (uint32_t)px * 37u + (uint32_t)py * 113u};
    float g[2];
    for (int k = 0; k < 2; ++k) {
        uint32_t v = (n[k] << 13) ^ n[k];
        v = v * (v * v * 15731u + 789221u) + 1376312589u;
        g[k] = -1.0f + 2.0f * (float)(int32_t)(v & 0x0fffffffu) / (float)0x0fffffff;
    }
    gx = g[0];
    gy = g[1];
}

// value and derivatives of gradient noise at (px, py)
void noised(float px, float py, float& val, float& ddx, float& ddy) {
    float flx = std::floor(px), fly = std::floor(py);
    int32_t ix = (int32_t)flx, iy = (int32_t)fly;
    float fx = px - flx, fy = py - fly;
    float ux = fx * fx * fx * (fx * (fx * 6.0f - 15.0f) + 10.0f);
    float uy = fy * fy * fy * (fy * (fy * 6.0f - 15.0f) + 10.0f);
    float dux = 30.0f * fx * fx * (fx * (fx - 2.0f) + 1.0f);
    float duy = 30.0f * fy * fy * (fy * (fy - 2.0f) + 1.0f);
    float gax, gay, gbx, gby, gcx, gcy, gdx, gdy;
    hash2(ix, iy, gax, gay);
    hash2(ix + 1, iy, gbx, gby);
    hash2(ix, iy + 1, gcx, gcy);
    hash2(ix + 1, iy + 1, gdx, gdy);
    float va = gax * (fx - 0.0f) + gay * (fy - 0.0f);
    float vb = gbx * (fx - 1.0f) + gby * (fy - 0.0f);
    float vc = gcx * (fx - 0.0f) + gcy * (fy - 1.0f);
    float vd = gdx * (fx - 1.0f) + gdy * (fy - 1.0f);
    float k = va - vb - vc + vd;
    float uxy = ux * uy;
    val = va + ux * (vb - va) + uy * (vc - va) + uxy * k;
    ddx = gax + ux * (gbx - gax) + uy * (gcx - gax) + uxy * (gax - gbx - gcx + gdx) + dux * (uy * k + vb - va);
    ddy = gay + ux * (gby - gay) + uy * (gcy - gay) + uxy * (gay - gby - gcy + gdy) + duy * (ux * k + vc - va);
}

float perlfbm(float vx, float vy, const FbmOpts& o) {
    vx += o.seed * 100.0f;
    vy += o.seed * 100.0f;
    float result = 0.0f, amp = 1.0f, freq = 1.0f, maximum = amp;
    for (int i = 0; i < o.octaves && i < 30; ++i) {  // MAX_FBM_ITERATIONS
        float val, dx, dy;
        noised(vx * freq * o.scale, vy * freq * o.scale, val, dx, dy);
        float v = (val + 1.0f) / 2.0f;
        if (o.turbulence) v = std::fabs(v);
        if (o.turbulence && o.ridge) v = 1.0f - v;
        result += v * amp;
        freq *= o.lacunarity;
        amp *= o.persistance;
        maximum += amp;
    }
    return redistribute(result, o.redistribution) / maximum;
}

float erosion_perlfbm(float vx, float vy, const FbmOpts& o) {
    vx += o.seed * 100.0f;
    vy += o.seed * 100.0f;
    float result = 0.0f, amp = 1.0f, freq = 1.5f, maximum = amp, sx = 0.0f, sy = 0.0f;
    for (int i = 0; i < o.octaves && i < 30; ++i) {  // MAX_FBM_ITERATIONS
        float val, dx, dy;
        noised(vx * freq * o.scale, vy * freq * o.scale, val, dx, dy);
        if (o.turbulence) { val = std::fabs(val); dx = std::fabs(dx); dy = std::fabs(dy); }
        if (o.turbulence && o.ridge) { val = 1.0f - val; dx = 1.0f - dx; dy = 1.0f - dy; }
        sx += dx;
        sy += dy;
        float v = (val + 1.0f) / 2.0f;
        result += v * amp / (1.0f + (sx * sx + sy * sy));
        freq *= o.lacunarity;
        amp *= o.persistance;
        maximum += amp;
    }
    return redistribute(result, o.redistribution) / maximum;
}

void heightmap_cell(const MapSettings& cfg, int x, int y, int n, float& rock, float& dirt) {
    const float fx = (float)x, fy = (float)y;
    const float uvx = fx / (float)n, uvy = fy / (float)n;
    const FbmOpts opts{cfg.seed, cfg.persistance, cfg.lacunarity, cfg.scale, 1.0f, cfg.octaves, false, false};
    float dsx = 1.0f, dsy = 1.0f;
    const float ws = cfg.domain_warp_scale;
    if (cfg.domain_warp != 0) {
        dsx = perlfbm(fx + 2.3f, fy + 2.9f, opts);
        dsy = perlfbm(fx - 3.1f, fy - 4.3f, opts);
        if (cfg.domain_warp == 2) {
            float ax = perlfbm(fx + ws * dsx - 5.7f, fy + ws * dsy + 27.9f, opts);
            float ay = perlfbm(fx + ws * dsx + 11.5f, fy + ws * dsy - 23.7f, opts);
            dsx = ax;
            dsy = ay;
        }
    }
    float val = erosion_perlfbm(fx + ws * dsx, fy + ws * dsy, opts);
    float hm = cfg.height_mult;
    if (cfg.uplift != 0) {
        const FbmOpts up_opts{cfg.seed, cfg.persistance, cfg.lacunarity, cfg.scale / cfg.uplift_scale, 1.0f,
                              cfg.octaves, true, true};
        float up = sfbm(fx - 7.3f, fy + 19.9f, up_opts);
        if (cfg.mask_exp != 0) hm += 2.5f;
        hm += 1.0f;
        val *= up;
    }
    if (cfg.mask_round != 0) {
        if (cfg.mask_exp != 0) hm += 16.0f;
        float ax = uvx - 0.5f, ay = uvy - 0.5f;
        float v = 1.0f - (ax * ax + ay * ay + 0.75f);
        val = val * gmaxf(0.0f, v * 1.0f);
    }
    if (cfg.mask_exp != 0) {
        hm += 2.0f;
        val = val * (std::exp(val) - 1.0f) / 1.718f;
    }
    if (cfg.mask_power != 0) {
        hm += 1.25f;
        if (cfg.mask_exp != 0) hm += 2.0f;
        float b = val + 0.5f;
        val = val * (((b * b * b - 0.125f) / 3.25f) * 0.55f + 0.45f);
    }
    if (cfg.mask_slope != 0) val = 0.25f * val + 0.75f * (val * uvx * uvy);
    val = val + (float)(4u * cfg.mask_round) * val;
    if (cfg.terrace > 0) {
        float step = 1.0f / ((float)cfg.terrace * hm);
        float lol = std::floor(val / step);
        float t = cfg.terrace_scale;
        val = (t * lol * step) + val * (1.0f - t);
    }
    rock = gminf(cfg.max_height, val * cfg.max_height * hm);
    dirt = (perlfbm(fx + 13.7f, fy + 27.1f, opts) + 1.5f) * cfg.max_dirt;
}

}  // namespace

extern "C" {

// glsl/heightmap.glsl main: rock and dirt of an n x n map
void hgo_ref_heightmap(const void* map_settings, int n, float* rock, float* dirt) {
    const MapSettings& cfg = *static_cast<const MapSettings*>(map_settings);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x) heightmap_cell(cfg, x, y, n, rock[(size_t)y * n + x], dirt[(size_t)y * n + x]);
}

// glsl/rain.glsl main: the water increment of every cell, from the total
// height (rock + dirt + water) and the frame time
void hgo_ref_rain(int n, const float* total, float time, float amount, float mountain_thresh, float mountain_multip,
                  float drops, float max_height, float* incr_out) {
    const FbmOpts opts{gfract(time * 1.372914227e3f) * 1000.0f, 0.5f, 2.0f, drops, 1.0f, 8, false, false};
#pragma omp parallel for schedule(static)
    for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x) {
            size_t i = (size_t)y * n + x;
            float r = gmaxf(0.0f, sfbm((float)x, (float)y, opts));
            float incr = amount * r;
            float mountain = total[i] - max_height * mountain_thresh;
            if (mountain > 0.0f) incr += mountain * mountain_multip * r / ((1.0f - mountain_thresh) * max_height);
            incr_out[i] = incr;
        }
}

float hgo_ref_rain_cell(int x, int y, float total, float time, float amount, float mountain_thresh,
                        float mountain_multip, float drops, float max_height) {
    const FbmOpts opts{gfract(time * 1.372914227e3f) * 1000.0f, 0.5f, 2.0f, drops, 1.0f, 8, false, false};
    float r = gmaxf(0.0f, sfbm((float)x, (float)y, opts));
    float incr = amount * r;
    float mountain = total - max_height * mountain_thresh;
    if (mountain > 0.0f) incr += mountain * mountain_multip * r / ((1.0f - mountain_thresh) * max_height);
    return incr;
}

float hgo_ref_simplex(float x, float y) { return simplex(x, y); }

void hgo_ref_noised(float x, float y, float* out3) { noised(x, y, out3[0], out3[1], out3[2]); }

}  // extern "C"
