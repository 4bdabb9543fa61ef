// Per-cell arithmetic of the grid-erosion step, shared by every kernel.
//
// Each function is the body of one GLSL pass for ONE cell, with the
// neighbourhood passed in as values, so the per-pass kernels, the fused
// kernel and the fused kernel's out-of-tile fallback evaluate exactly the same
// float expression tree (one rounding per operation; the library is built
// with -fmad=false so nvcc does not contract a*b+c).  Each function cites the
// GLSL lines it implements (paths inside the hydro-gen project).
//
// The world is the single-material form of the reference model: rock in
// heightmap.r, an empty dirt layer (heightmap.g == 0, sedimap.g == 0,
// Kconv == 0, Kspeed[1] == 0), which the reference evaluates with the dirt
// terms vanishing exactly; the comments below say where that is used.
#pragma once
#include <cstdint>

namespace hg {

// GLSL built-ins with GLSL's operand order (min(x,y) = y<x?y:x, ...).
__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
__device__ __forceinline__ float gmix(float x, float y, float a) { return x * (1.0f - a) + y * a; }

// out-of-range height used by the flux and thermal passes
// (glsl/hydro_flux.glsl:36, glsl/thermal_erosion.glsl:23): 999999999999.0 as float
constexpr float FAR_HEIGHT = 999999995904.0f;

// Single-precision arctangent (coefficients from oracle/fit_atan.py, a Lawson
// minimax fit): three branches keep the
// polynomial argument within |u| <= tan(pi/8),
//   x <= tan(pi/8): poly(x);  x <= tan(3pi/8): pi/4 + poly((x-1)/(x+1));
//   else pi/2 - poly(1/x);    poly(u) = u + u*(s*P(s)), s = u*u.
// Max error 2.5 ulp; monotone non-decreasing on x >= 0 (checked over every
// positive float).
__device__ __forceinline__ float poly_atan_core(float u) {
    const float c0 = -3.333333135e-01f, c1 = 1.999990344e-01f, c2 = -1.428200752e-01f,
                c3 = 1.104469076e-01f, c4 = -8.476266265e-02f, c5 = 4.744043201e-02f;
    float s = __fmul_rn(u, u);
    float p = c5;
    p = __fadd_rn(__fmul_rn(p, s), c4);
    p = __fadd_rn(__fmul_rn(p, s), c3);
    p = __fadd_rn(__fmul_rn(p, s), c2);
    p = __fadd_rn(__fmul_rn(p, s), c1);
    p = __fadd_rn(__fmul_rn(p, s), c0);
    return __fadd_rn(u, __fmul_rn(u, __fmul_rn(s, p)));
}
// The three branches share one division and one polynomial evaluation
// (lanes of a warp taking different branches do not repeat them).
__device__ __forceinline__ float poly_atanf(float x) {
    const float ax = fabsf(x);
    const bool mid = ax > 0.414213562f && ax <= 2.41421356f;
    const bool big = ax > 2.41421356f;
    float u = ax;
    if (mid || big) u = __fdiv_rn(mid ? __fsub_rn(ax, 1.0f) : 1.0f, mid ? __fadd_rn(ax, 1.0f) : ax);
    const float p = poly_atan_core(u);
    float r = p;
    if (mid) r = __fadd_rn(0.785398163f, p);
    else if (big) r = __fsub_rn(1.57079637f, p);
    return copysignf(r, x);
}

// Correctly rounded a / b from y = RN(1/b), two correction steps after the
// product a*y (P. Markstein, "Computation of elementary functions on the IBM
// RISC System/6000 processor", IBM J. Res. Develop. 34(1), 1990): q0 = RN(a*y)
// lies within 2 ulp of a/b, the first correction brings it within 1 ulp, and
// with y within half an ulp of 1/b Markstein's theorem makes the second
// correction the correctly rounded quotient.  Holds while no product
// overflows and no residual underflows: callers keep a at 0 or in
// [2^-80, 2^80] and b in [2^-30, 2^40].
__device__ __forceinline__ float div_recip(float a, float b, float y) {
    float q = __fmul_rn(a, y);
    float r = __fmaf_rn(-q, b, a);
    q = __fmaf_rn(r, y, q);
    r = __fmaf_rn(-q, b, a);
    return __fmaf_rn(r, y, q);
}
constexpr float SQRT2_F = 1.41421354f;
constexpr float RCP_SQRT2_F = 0x1.6a09e6p-1f;  // RN(1 / SQRT2_F)

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers:
// as easy as 1, 2, 3", SC'11) ---------------------------------------------------
__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
        uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// Rain settings resolved for one step.
struct RainStep {
    int active;          // this step rains
    int bernoulli;       // 0 uniform, 1 Bernoulli
    float amount;
    uint32_t threshold;  // Bernoulli: rain when the Philox word < threshold
    uint32_t seed_lo, seed_hi, terrain_id;
    uint32_t step;       // 1-based step number (Philox counter word 2)
};

// One Philox call covers the four cells x0..x0+3 (x0 % 4 == 0):
// counter (x0/4, y, step, terrain), key (seed).  Cell x uses word x % 4.
__device__ __forceinline__ void rain_words4(const RainStep& r, int x0, int y, uint32_t out[4]) {
    out[0] = (uint32_t)x0 >> 2; out[1] = (uint32_t)y; out[2] = r.step; out[3] = r.terrain_id;
    philox4x32_10(out, r.seed_lo, r.seed_hi);
}

// glsl/rain.glsl:48-53 with the workload's rain amount: water += incr.
__device__ __forceinline__ float rain_incr(const RainStep& r, uint32_t word) {
    if (!r.bernoulli) return r.amount;
    return word < r.threshold ? r.amount : 0.0f;
}

// ---- constants of one step -----------------------------------------------------
struct StepConsts {
    int n;
    float dt, G, EK;      // d_t, G, ENERGY_KEPT
    float Kc;
    float Kls0, Kld0;     // d_t*Ks[0], d_t*Kd[0] (rock)
    float Kls1, Kld1;     // d_t*Ks[1], d_t*Kd[1] (empty dirt layer)
    float Ks0;            // Ks[0] when no per-cell field is set
    const float* ks_field;  // per-cell Ks[0] or nullptr
    float evap;           // 1 - Ke*d_t
    float Kalpha0, Kspeed0;
    int thermal;          // thermal layer-0 passes enabled (Kspeed[0] != 0)
    float talus_x_cross;  // smallest positive slope whose poly_atanf exceeds Kalpha0
    float talus_b_diag;   // smallest positive height drop whose diagonal slope does
    int fast_div;         // both thresholds >= 2^-30: outflow quotients by div_recip
    float smooth_m;       // smoothing weight clamp(Kspeed[1]*d_t, 0, 1); 0: the pass is the identity
    // two-layer worlds (rock + dirt)
    float Ks1;            // Ks[1]
    float Kconv;          // sediment conversion rock -> dirt
    float Kalpha1, Kspeed1;
    int row_lo, row_hi;   // the per-pass kernels compute rows [row_lo, row_hi) only (a row slab)
};

// Layer 1's talus thresholds (as talus_x_cross, talus_b_diag, fast_div of
// layer 0; kept out of StepConsts, which batch launches carry per terrain).
struct Talus1 {
    float x_cross, b_diag;
    int fast_div;
};

// ---- hydro_flux, glsl/hydro_flux.glsl:77-166 -------------------------------------
// w* are neighbour totals (rock + water after rain; FAR_HEIGHT outside the
// grid), in* the neighbours' old flux facing this cell (left.fR, right.fL,
// top.fB, bottom.fT; 0 outside).  The 1-layer total is rock + water: the
// reference's (r + d2) + g with g == 0 is the same float.
struct FluxOut { float fl, fr, ft, fb, d2, u, v, vz; };

__device__ __forceinline__ FluxOut cell_flux(const StepConsts& c, int x, int y,
                                             float w_c, float d1,
                                             float fl, float fr, float ft, float fb,
                                             float wl, float wr, float wt, float wb,
                                             float inl, float inr, float int_, float inb,
                                             bool border = true) {
    FluxOut o;
    // :88-92 total height differences; :100-107 new outflow (A == L == 1, the
    // products and quotients by 1 are exact and dropped)
    float dhl = w_c - wl, dhr = w_c - wr, dht = w_c - wt, dhb = w_c - wb;
    o.fl = gmax(0.0f, c.EK * fl + c.dt * (c.G * dhl));
    o.fr = gmax(0.0f, c.EK * fr + c.dt * (c.G * dhr));
    o.ft = gmax(0.0f, c.EK * ft + c.dt * (c.G * dht));
    o.fb = gmax(0.0f, c.EK * fb + c.dt * (c.G * dhb));
    // :110-119 closed boundaries (callers that never see the grid edge pass
    // border = false)
    if (border) {
        if (x <= 0) o.fl = 0.0f;
        else if (x >= c.n - 1) o.fr = 0.0f;
        if (y <= 0) o.fb = 0.0f;
        else if (y >= c.n - 1) o.ft = 0.0f;
    }
    // :121-127 scale outflow to the available water
    float sum_in = inl + inr + int_ + inb;
    float sum_out = o.fl + o.fr + o.ft + o.fb;
    // K = min(1, d1 / den).  d1 >= den means the exact quotient is >= 1 (or
    // 0/0, inf/inf: NaN, which GLSL's min also maps to 1), so K = 1 without
    // dividing; otherwise the division decides.
    float den = sum_out * c.dt;
    float K = d1 >= den ? 1.0f : gmin(1.0f, d1 / den);
    o.fl *= K; o.fr *= K; o.ft *= K; o.fb *= K;
    sum_out *= K;
    // :133-134 water update
    float d_volume = c.dt * (sum_in - sum_out);
    o.d2 = gmax(0.0f, d1 + d_volume);
    // :144-161 velocity from the OLD flux field
    o.vz = d1 + o.d2;
    if (o.vz > 0.0f) {
        o.u = (inl - fl + fr - inr) / o.vz;
        o.v = (inb - fb + ft - int_) / o.vz;
    } else {
        o.u = 0.0f; o.v = 0.0f;
    }
    return o;
}

// ---- hydro_erosion, glsl/hydro_erosion.glsl:23-92 --------------------------------
// b* are the neighbours' rock heights (0 outside the grid: imageLoad of an
// out-of-range texel).  With the dirt channel at 0, (r.r + r.g) - l.r - l.g
// equals r.r - l.r exactly.
__device__ __forceinline__ void cell_erosion(const StepConsts& c, float Kls0, float u, float v, float vz,
                                             float& b, float& s,
                                             float br, float bl, float bb, float bt) {
    // :45-52 erosion speed, faded out in very shallow water
    float len = sqrtf(u * u + v * v);
    float ero_vel = len;
    if (vz < 1e-3f) {
        float dd = gmax(5e-4f, vz);
        float t = gclamp((dd - 1e-3f) / (5e-4f - 1e-3f), 0.0f, 1.0f);
        t = t * t * (3.0f - 2.0f * t);
        ero_vel = gmix(len, 0.0f, t);
    }
    // :23-35, :56-57 terrain normal -> sin of the tilt
    float dx = br - bl;
    float dz = bt - bb;
    float cx = dx * 2.0f - 0.0f * dz;
    float cy = 0.0f * 0.0f - 2.0f * 2.0f;
    float cz = 2.0f * dz - dx * 0.0f;
    float len3 = sqrtf(cx * cx + cy * cy + cz * cz);
    float ny = cy / len3;
    float sin_a = fabsf(sqrtf(1.0f - ny * ny));
    // :58-83 layer loop.  Dirt layer (i = 1) first: with no dirt and no dirt
    // sediment it dissolves Kls1*c, hands all of it back and continues with
    // cap == 0, unless Kls1*c rounds to 0, in which case the reference breaks
    // out of the loop before the rock layer.
    float cap = 0.0f;
    float cc = gmax(0.0f, c.Kc * gmax(0.02f, sin_a) * ero_vel - cap);
    if (cc > 0.0f && !(c.Kls1 * cc > 0.0f)) return;
    // rock layer (i = 0)
    if (cc > s) {
        float delta = Kls0 * (cc - s);
        b = b - delta;
        s = s + delta;
        if (b < 0.0f) {  // cap += old terrain is dropped: no later layer reads it
            s = s + b;
            b = 0.0f;
        }
    } else {
        float delta = c.Kld0 * (s - cc);
        b = b + delta;
        s = s - delta;
    }
    // :84-88 conversion with Kconv == 0 leaves s unchanged
}

// Two-layer form (rock r, dirt g; rock sediment s0, dirt sediment s1):
// the shader's layer loop from dirt down to rock and the s0 -> s1
// conversion.  Neighbours' heights are (rock, dirt) pairs, 0 outside.
__device__ __forceinline__ void cell_erosion2(const StepConsts& c, float Kls0, float u, float v, float vz,
                                              float& r, float& g, float& s0, float& s1,
                                              float rr, float rg, float lr, float lg,
                                              float tr, float tg, float br, float bg) {
    float len = sqrtf(u * u + v * v);
    float ero_vel = len;
    if (vz < 1e-3f) {
        float dd = gmax(5e-4f, vz);
        float t = gclamp((dd - 1e-3f) / (5e-4f - 1e-3f), 0.0f, 1.0f);
        t = t * t * (3.0f - 2.0f * t);
        ero_vel = gmix(len, 0.0f, t);
    }
    // :23-35 (r.r + r.g) - l.r - l.g, likewise along y
    float dx = rr + rg - lr - lg;
    float dz = tr + tg - br - bg;
    float cx = dx * 2.0f - 0.0f * dz;
    float cy = 0.0f * 0.0f - 2.0f * 2.0f;
    float cz = 2.0f * dz - dx * 0.0f;
    float len3 = sqrtf(cx * cx + cy * cy + cz * cz);
    float ny = cy / len3;
    float sin_a = fabsf(sqrtf(1.0f - ny * ny));
    float terr[2] = {r, g}, sed[2] = {s0, s1};
    const float Kls[2] = {Kls0, c.Kls1}, Kld[2] = {c.Kld0, c.Kld1};
    float cap = 0.0f;
#pragma unroll
    for (int i = 1; i >= 0; --i) {
        float cc = gmax(0.0f, c.Kc * gmax(0.02f, sin_a) * ero_vel - cap);
        if (cc > sed[i]) {
            float old = terr[i];
            terr[i] = terr[i] - Kls[i] * (cc - sed[i]);
            sed[i] = sed[i] + Kls[i] * (cc - sed[i]);
            if (terr[i] < 0.0f) {
                sed[i] = sed[i] + terr[i];
                terr[i] = 0.0f;
                cap = cap + old;
            } else {
                break;
            }
        } else {
            terr[i] = terr[i] + Kld[i] * (sed[i] - cc);
            sed[i] = sed[i] - Kld[i] * (sed[i] - cc);
        }
    }
    // :84-88 conversion of rock sediment into dirt sediment
    float conv = sed[0] * c.Kconv * c.dt;
    sed[1] = sed[1] + conv;
    sed[0] = sed[0] - conv;
    r = terr[0]; g = terr[1]; s0 = sed[0]; s1 = sed[1];
}

// ---- sediment_transport, glsl/sediment_transport.glsl:66-93 ----------------------
// Back-trace point of the semi-Lagrangian step (:70, clamp :26-29).
__device__ __forceinline__ void backtrace(const StepConsts& c, int x, int y, float u, float v,
                                          float& px, float& py) {
    float maxc = (float)(c.n - 1);
    px = gclamp((float)x - u * c.dt, 0.0f, maxc);
    py = gclamp((float)y - v * c.dt, 0.0f, maxc);
}

// img_bilinear, glsl/img_interpolation.glsl:3-22: s00 at (ix, iy), s10 at
// (ix+1, iy), s01 at (ix, iy+1), s11 at (ix+1, iy+1), out-of-range taps 0.
__device__ __forceinline__ float bilinear_mix(float px, float py, float s00, float s10, float s01, float s11) {
    float fx = px - floorf(px), fy = py - floorf(py);
    float v1 = gmix(s00, s10, fx);
    float v2 = gmix(s01, s11, fx);
    return gmix(v1, v2, fy);
}

// ---- thermal_erosion (layer 0), glsl/thermal_erosion.glsl:28-109 ------------------
// Outflow of one cell toward its 8 neighbours, order L, R, T, B, LT, RT, LB, RB
// (cross (-1,0),(1,0),(0,1),(0,-1); diagonal (-1,1),(1,1),(-1,-1),(1,-1)).
// nb[k] is the neighbour's rock (FAR_HEIGHT outside the grid).  Returns the
// mask of marked directions and S and bk such that the outflow toward a
// marked direction k is (S * dh_k) / bk.
struct ThermalOut { float S, bk; uint32_t mask; };

// Faithful form: one arctangent per downhill direction, as in the shader,
// for the drops dh[] (summed over the layers up to this one) and the layer's
// own height `terr`, talus angle and slippage rate.
__device__ __forceinline__ ThermalOut cell_thermal_dh(float dt, float Kalpha, float Kspeed, float terr,
                                                      const float dh[8]) {
    float H = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (dh[k] > H) H = dh[k];
    H = gmin(terr, H);
    ThermalOut o{0.0f, 0.0f, 0u};
    float sharp = 1.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        float bb = dh[k];
        if (bb <= 0.0f) continue;
        float slope = k < 4 ? bb : bb / 1.41421354f;  // d = L (cross) or L*sqrt(2)
        float alph = poly_atanf(slope);
        if (alph > Kalpha) {
            float newsh = 1.0f + alph - Kalpha;
            if (newsh > sharp) sharp = newsh;
            o.bk += bb;
            o.mask |= 1u << k;
        }
    }
    sharp *= sharp * sharp;
    o.S = dt * Kspeed * sharp * H / 2.0f;  // a == L == 1
    return o;
}

// Layer 0 (rock): drops b - nb (the shader's 0 + (b - nb)).
__device__ __forceinline__ ThermalOut cell_thermal_ref(const StepConsts& c, float b, const float nb[8]) {
    float dh[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) dh[k] = b - nb[k];
    return cell_thermal_dh(c.dt, c.Kalpha0, c.Kspeed0, b, dh);
}

// The shader's outflows with one arctangent per cell, written to o[8].
// poly_atanf is monotone non-decreasing on x >= 0 (checked over every
// positive float), so "poly_atanf(slope) > Kalpha0" is "slope >=
// talus_x_cross" (diagonal: "drop >= talus_b_diag", division rounding being
// monotone too; both thresholds are positive, so a marked drop is > 0), and
// the largest marked sharpness is that of the steepest marked slope.  The
// quotients S*dh/bk share their divisor: with the operands in div_recip's
// range they come from one reciprocal, else from IEEE division; either way
// they are the correctly rounded quotients of the shader's expression.
__device__ __forceinline__ void cell_thermal_outflows_dh(float dt, float Kalpha, float Kspeed, float x_cross,
                                                        float b_diag, int fast_div, float terr, const float dh[8],
                                                        float o[8]) {
    // H only matters when a direction is marked, i.e. some drop is >= a
    // positive threshold: then the shader's "if (dh > H) H = dh" from 0 and
    // fmaxf agree (NaN drops are skipped by both)
    float H = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) H = fmaxf(H, dh[k]);
    H = gmin(terr, H);
    // marked drops (0 where unmarked): sums and maxima over the marked set
    float dm[8], bk = 0.0f, max_cross = 0.0f, max_diag = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        dm[k] = dh[k] >= (k < 4 ? x_cross : b_diag) ? dh[k] : 0.0f;
        bk += dm[k];  // + 0 leaves the sum's bits unchanged (it starts at +0)
        if (k < 4) max_cross = fmaxf(max_cross, dm[k]);
        else max_diag = fmaxf(max_diag, dm[k]);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) o[k] = 0.0f;
    if (!(bk > 0.0f)) return;  // no marked direction (marked drops are > 0)
    bool fast = fast_div && bk <= 0x1p40f;  // then max_diag is 0 or in [2^-30, 2^40]
    const float sd = fast ? div_recip(max_diag, SQRT2_F, RCP_SQRT2_F) : max_diag / SQRT2_F;
    const float alph = poly_atanf(fmaxf(max_cross, sd));
    float sharp = 1.0f;
    const float newsh = 1.0f + alph - Kalpha;
    if (newsh > sharp) sharp = newsh;
    sharp *= sharp * sharp;
    const float S = dt * Kspeed * sharp * H / 2.0f;  // a == L == 1
    fast = fast && S >= 0x1p-50f && S <= 0x1p40f;
    if (fast) {
        // S > 0: an unmarked direction's dividend S * 0 is +0 and its
        // quotient +0, the shader's 0
        const float y = __frcp_rn(bk);
#pragma unroll
        for (int k = 0; k < 8; ++k) o[k] = div_recip(S * dm[k], bk, y);
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (dm[k] != 0.0f) o[k] = S * dh[k] / bk;
    }
}

// Layer 0 (rock): drops b - nb[k], H capped by b.
__device__ __forceinline__ void cell_thermal_outflows(const StepConsts& c, float b, const float nb[8], float o[8]) {
    float dh[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) dh[k] = b - nb[k];
    cell_thermal_outflows_dh(c.dt, c.Kalpha0, c.Kspeed0, c.talus_x_cross, c.talus_b_diag, c.fast_div, b, dh, o);
}

// Layer 1 (dirt) of a two-layer world: drops summed over rock and dirt,
// (0 + (r - nr)) + (g - ng), H capped by the dirt height g.
__device__ __forceinline__ void cell_thermal_outflows1(const StepConsts& c, const Talus1& t, const float dh[8],
                                                       float g, float o[8]) {
    cell_thermal_outflows_dh(c.dt, c.Kalpha1, c.Kspeed1, t.x_cross, t.b_diag, t.fast_div, g, dh, o);
}

// ---- two cells at once: paired FP32 arithmetic ----------------------------------
// sm_100-class GPUs issue two independent IEEE single-precision adds,
// multiplies or fused multiply-adds as one f32x2 instruction.  Each lane
// rounds exactly as the scalar operation, so two cells evaluated in lanes .x
// and .y keep the scalar cells' bits while the pair costs one issue slot.
__device__ __forceinline__ float2 pf(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
        "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
// The multiply is a fused multiply-add of -0: a * b + (-0) is a * b
// rounded once, signed zeros included.  The -0 pair sits in constant
// memory, so the compiler cannot turn it back into a multiply instruction:
// at -O3 ptxas contracts an f32x2 multiply that feeds an f32x2 add into one
// fused multiply-add, even with .rn and --fmad=false (measured: a
// two-product mix differed from the scalar one in a third of the lanes),
// while a fused multiply-add feeding an add stays two roundings.
static __constant__ float2 kNegZero2 = {-0.0f, -0.0f};
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return fma2(a, b, kNegZero2); }
// a - b as b * (-1) + a: the product is exact, so this is one rounding of
// a - b (signed zeros included)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return fma2(b, make_float2(-1.0f, -1.0f), a); }

// div_recip on two lanes with nb = -b: fma(q, -b, a) is fma(-q, b, a)
// exactly (the product's sign moves, nothing rounds differently).
__device__ __forceinline__ float2 div_recip2(float2 a, float2 nb, float2 y) {
    float2 q = mul2(a, y);
    float2 r = fma2(q, nb, a);
    q = fma2(r, y, q);
    r = fma2(q, nb, a);
    return fma2(r, y, q);
}

// poly_atanf of two non-negative arguments: the reduction's division runs
// per lane, the polynomial on the pair.
__device__ __forceinline__ float2 poly_atanf2(float2 x) {
    const float c0 = -3.333333135e-01f, c1 = 1.999990344e-01f, c2 = -1.428200752e-01f,
                c3 = 1.104469076e-01f, c4 = -8.476266265e-02f, c5 = 4.744043201e-02f;
    const bool midx = x.x > 0.414213562f && x.x <= 2.41421356f, bigx = x.x > 2.41421356f;
    const bool midy = x.y > 0.414213562f && x.y <= 2.41421356f, bigy = x.y > 2.41421356f;
    float2 u = x;
    if (midx || bigx) u.x = __fdiv_rn(midx ? __fsub_rn(x.x, 1.0f) : 1.0f, midx ? __fadd_rn(x.x, 1.0f) : x.x);
    if (midy || bigy) u.y = __fdiv_rn(midy ? __fsub_rn(x.y, 1.0f) : 1.0f, midy ? __fadd_rn(x.y, 1.0f) : x.y);
    const float2 s = mul2(u, u);
    float2 p = pf(c5);
    p = add2(mul2(p, s), pf(c4));
    p = add2(mul2(p, s), pf(c3));
    p = add2(mul2(p, s), pf(c2));
    p = add2(mul2(p, s), pf(c1));
    p = add2(mul2(p, s), pf(c0));
    p = add2(u, mul2(u, mul2(s, p)));
    const float2 pm = add2(pf(0.785398163f), p), pb = sub2(pf(1.57079637f), p);
    return make_float2(midx ? pm.x : bigx ? pb.x : p.x, midy ? pm.y : bigy ? pb.y : p.y);
}

// cell_thermal_outflows_dh for two cells (lanes .x, .y) with the same
// operations per lane; dm holds the drops on entry and is overwritten with
// the marked drops (0 where unmarked: a marked drop equals its drop, so the
// scalar fallback's S * dh reads it from there).  A lane with no marked
// direction keeps its zeros; it runs the paired quotients on a divisor of 1
// and a dividend of +0, whose quotient is +0, so the pair stays on one path.
// Lanes whose operands leave div_recip's range take the scalar path of
// cell_thermal_outflows_dh.
__device__ __forceinline__ void cell_thermal_outflows_dh2(float dt, float Kalpha, float Kspeed, float x_cross,
                                                          float b_diag, int fast_div, float2 terr, float2 dm[8],
                                                          float2 o[8]) {
    float Hx = 0.0f, Hy = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        Hx = fmaxf(Hx, dm[k].x);
        Hy = fmaxf(Hy, dm[k].y);
    }
    const float2 H = make_float2(gmin(terr.x, Hx), gmin(terr.y, Hy));
    float2 bk = pf(0.0f);
    float mcx = 0.0f, mcy = 0.0f, mdx = 0.0f, mdy = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const float t = k < 4 ? x_cross : b_diag;
        dm[k] = make_float2(dm[k].x >= t ? dm[k].x : 0.0f, dm[k].y >= t ? dm[k].y : 0.0f);
        bk = add2(bk, dm[k]);
        if (k < 4) {
            mcx = fmaxf(mcx, dm[k].x);
            mcy = fmaxf(mcy, dm[k].y);
        } else {
            mdx = fmaxf(mdx, dm[k].x);
            mdy = fmaxf(mdy, dm[k].y);
        }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) o[k] = pf(0.0f);
    const bool mx = bk.x > 0.0f, my = bk.y > 0.0f;
    if (!mx && !my) return;
    bool fx = fast_div && bk.x <= 0x1p40f, fy = fast_div && bk.y <= 0x1p40f;
    float2 sd;
    if ((fx || !mx) && (fy || !my)) {
        sd = div_recip2(make_float2(mdx, mdy), pf(-SQRT2_F), pf(RCP_SQRT2_F));
    } else {
        sd.x = fx ? div_recip(mdx, SQRT2_F, RCP_SQRT2_F) : mdx / SQRT2_F;
        sd.y = fy ? div_recip(mdy, SQRT2_F, RCP_SQRT2_F) : mdy / SQRT2_F;
    }
    const float2 alph = poly_atanf2(make_float2(fmaxf(mcx, sd.x), fmaxf(mcy, sd.y)));
    const float2 newsh = sub2(add2(pf(1.0f), alph), pf(Kalpha));
    float2 sharp = make_float2(newsh.x > 1.0f ? newsh.x : 1.0f, newsh.y > 1.0f ? newsh.y : 1.0f);
    sharp = mul2(sharp, mul2(sharp, sharp));
    // dt * Kspeed * sharp * H / 2 (a == L == 1); halving is exact either way
    const float2 S = mul2(mul2(mul2(pf(dt * Kspeed), sharp), H), pf(0.5f));
    fx = fx && S.x >= 0x1p-50f && S.x <= 0x1p40f;
    fy = fy && S.y >= 0x1p-50f && S.y <= 0x1p40f;
    if ((fx || !mx) && (fy || !my)) {
        const float2 b = make_float2(mx ? bk.x : 1.0f, my ? bk.y : 1.0f);
        const float2 y = make_float2(__frcp_rn(b.x), __frcp_rn(b.y));
        const float2 nb = make_float2(-b.x, -b.y);
        const float2 S2 = make_float2(mx ? S.x : 0.0f, my ? S.y : 0.0f);
#pragma unroll
        for (int k = 0; k < 8; ++k) o[k] = div_recip2(mul2(S2, dm[k]), nb, y);
        return;
    }
    if (mx) {
        if (fx) {
            const float y = __frcp_rn(bk.x);
#pragma unroll
            for (int k = 0; k < 8; ++k) o[k].x = div_recip(S.x * dm[k].x, bk.x, y);
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (dm[k].x != 0.0f) o[k].x = S.x * dm[k].x / bk.x;
        }
    }
    if (my) {
        if (fy) {
            const float y = __frcp_rn(bk.y);
#pragma unroll
            for (int k = 0; k < 8; ++k) o[k].y = div_recip(S.y * dm[k].y, bk.y, y);
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (dm[k].y != 0.0f) o[k].y = S.y * dm[k].y / bk.y;
        }
    }
}

// Layer 0 (rock) for two cells: drops b - nb[k] (nb is overwritten).
__device__ __forceinline__ void cell_thermal_outflows2(const StepConsts& c, float2 b, float2 nb[8], float2 o[8]) {
#pragma unroll
    for (int k = 0; k < 8; ++k) nb[k] = sub2(b, nb[k]);
    cell_thermal_outflows_dh2(c.dt, c.Kalpha0, c.Kspeed0, c.talus_x_cross, c.talus_b_diag, c.fast_div, b, nb, o);
}

// backtrace + bilinear_mix for two cells at (x, y) and (x + 1, y): the
// back-trace points and the mix weights on the pair, the clamps, floors and
// tap indices per lane.
__device__ __forceinline__ void backtrace2(const StepConsts& c, int x, int y, float2 u, float2 v, float2& px,
                                           float2& py) {
    const float maxc = (float)(c.n - 1);
    const float2 tx = sub2(make_float2((float)x, (float)(x + 1)), mul2(u, pf(c.dt)));
    const float2 ty = sub2(pf((float)y), mul2(v, pf(c.dt)));
    px = make_float2(gclamp(tx.x, 0.0f, maxc), gclamp(tx.y, 0.0f, maxc));
    py = make_float2(gclamp(ty.x, 0.0f, maxc), gclamp(ty.y, 0.0f, maxc));
}
__device__ __forceinline__ float2 gmix2(float2 x, float2 y, float2 a) {
    return add2(mul2(x, sub2(pf(1.0f), a)), mul2(y, a));
}
__device__ __forceinline__ float2 bilinear_mix2(float2 px, float2 py, float2 s00, float2 s10, float2 s01,
                                                float2 s11) {
    const float2 fx = sub2(px, make_float2(floorf(px.x), floorf(px.y)));
    const float2 fy = sub2(py, make_float2(floorf(py.x), floorf(py.y)));
    return gmix2(gmix2(s00, s10, fx), gmix2(s01, s11, fx), fy);
}

// ---- thermal_transport (layer 0), glsl/thermal_transport.glsl:31-65 ----------------
// own[k]: this cell's outflow in direction order L,R,T,B,LT,RT,LB,RB;
// inflow: L.R, R.L, T.B, B.T, LT.RB, RT.LB, LB.RT, RB.LT (0 outside).
__device__ __forceinline__ float cell_thermal_apply(float b, const float own[8], const float in[8]) {
    float in_flux = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) in_flux += in[k];
    float sum = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) sum -= own[k];
    sum += in_flux;
    return b + sum;
}

// ---- smoothing, glsl/smoothing.glsl:22-103 (grid branch), rock channel -----------
// Interior cell with rock tr and neighbours lr, rr, tt (y+1), bt (y-1); border
// cells are copied by the caller.  With the dirt channel at 0 the dirt
// differences equal the rock differences (0 - 0 + d == d) and the dirt average
// is 0, so dirt stays exactly 0 and only rock changes: a local extremum along
// x or y moves toward its 4-neighbour mean by the weight m.
__device__ __forceinline__ float cell_smooth(float m, float tr, float lr, float rr, float tt, float bt) {
    float dl = tr - lr, dr = tr - rr, dt_ = tr - tt, db = tr - bt;
    float hdiff = fabsf((dl + dr + dt_ + db) / 4.0f);
    float xs = dl * dr, ys = dt_ * db;
    float nr = tr;
    if (((-dl > hdiff || -dr > hdiff) && xs > 0.0f) || ((-dt_ > hdiff || -db > hdiff) && ys > 0.0f))
        nr = (tr + lr + rr + tt + bt) / 5.0f;
    return m * nr + (1.0f - m) * tr;
}

// Two-layer smoothing (rock r, dirt g; neighbours left, right, top (y+1),
// bottom (y-1)): the dirt differences include the rock differences.
__device__ __forceinline__ void cell_smooth2(float m, float& tr, float& tg, float lr, float lg, float rr, float rg,
                                             float ttr, float ttg, float bbr, float bbg) {
    float dlr = tr - lr, dlg = tg - lg;
    dlg += dlr;
    float drr = tr - rr, drg = tg - rg;
    drg += drr;
    float dtr = tr - ttr, dtg = tg - ttg;
    dtg += dtr;
    float dbr = tr - bbr, dbg = tg - bbg;
    dbg += dbr;
    float g_hdiff = fabsf((dlg + drg + dtg + dbg) / 4.0f);
    float r_hdiff = fabsf((dlr + drr + dtr + dbr) / 4.0f);
    float xr = dlr * drr, xg = dlg * drg;
    float yr = dtr * dbr, yg = dtg * dbg;
    float nr = tr, ng = tg;
    if (((-dlr > r_hdiff || -drr > r_hdiff) && xr > 0.0f) || ((-dtr > r_hdiff || -dbr > r_hdiff) && yr > 0.0f))
        nr = (tr + lr + rr + ttr + bbr) / 5.0f;
    if (((-dlg > g_hdiff || -drg > g_hdiff) && xg > 0.0f) || ((-dtg > g_hdiff || -dbg > g_hdiff) && yg > 0.0f))
        ng = (tg + lg + rg + ttg + bbg) / 5.0f;
    tr = m * nr + (1.0f - m) * tr;
    tg = m * ng + (1.0f - m) * tg;
}

}  // namespace hg
