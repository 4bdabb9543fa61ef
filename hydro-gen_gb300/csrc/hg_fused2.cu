// Fused step of a two-layer (rock + dirt) world, the reference's own model,
// in three kernels per step instead of the nine per-pass launches:
//   k2f_hydro      rain -> hydro_flux -> hydro_erosion (both layers, Kconv)
//                  -> evaporation; 64 x 16 tiles, nine fields TMA-staged
//                  with a 4-column, 1-row halo
//   k2f_transport  sediment_transport of both sediment channels (one
//                  back-trace, two gathers from L2/HBM) and the rock talus
//                  pass (thermal_erosion/thermal_transport, layer 0) on the
//                  TMA-staged eroded rock
//   k2f_layer1     the dirt talus pass (layer 1: cumulative rock + dirt
//                  drops, capped by the dirt height) and smoothing of both
//                  channels, on rock and dirt staged with a 3-cell halo:
//                  outflows on the tile plus two rings, transport on the
//                  tile plus one ring, smoothing on the tile
// (src/erosion.cpp:158-200; glsl/hydro_flux.glsl, hydro_erosion.glsl,
// sediment_transport.glsl, thermal_erosion.glsl, thermal_transport.glsl,
// smoothing.glsl).  Per-cell arithmetic is the per-pass kernels' code, so
// the fused step equals them bit for bit.  The particle step
// (src/erosion.cpp:132-156) reuses the last two: the rock talus pass alone,
// then the dirt talus pass with smoothing's particle branch (momentum fold,
// water decay; glsl/smoothing.glsl:76-95).
#include "hg_internal.h"
#include "hg_tma.cuh"

namespace hg {

namespace {

constexpr int TW = 64, TH = 16, HX = 4, RW = TW + 2 * HX;  // 72
constexpr int NT = 256;                                    // threads per block
constexpr int GPR = TW / 4;                                // row groups per tile row
enum { F_B = 0, F_G, F_D, F_S0, F_S1, F_FL, F_FR, F_FT, F_FB, F_N };
constexpr int H_RH = TH + 2, H_BOX = RW * H_RH, H_RC = ((H_BOX + 31) / 32) * 32;
constexpr int T_RH = TH + 4, T_BOX = RW * T_RH;            // eroded rock, 2-row halo
constexpr int O_RH = TH + 2, O_C = RW * O_RH;              // rock outflows of the tile plus 1
constexpr int L_RH = TH + 6, L_BOX = RW * L_RH;            // layer-1 inputs, 3-row halo
constexpr int L_RC = ((L_BOX + 31) / 32) * 32;             // 128-byte aligned array stride
constexpr int P_W = TW + 4, P_H = TH + 4, P_C = P_W * P_H; // layer-1 outflows of the tile plus 2

__constant__ int f2_ox[8] = {-1, 1, 0, 0, -1, 1, -1, 1};
__constant__ int f2_oy[8] = {0, 0, 1, -1, 1, 1, -1, -1};

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float at4(const float4& v, int j) { return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w; }

struct HydroArgs {
    CUtensorMap maps[F_N];  // rock, dirt, water, sediment rock / dirt, fL, fR, fT, fB (72 x 18 boxes)
    StepConsts c;
    RainStep r;
    float *water, *fl, *fr, *ft, *fb, *u, *v;
    float *s0, *s1;      // eroded sediment (rock, dirt)
    float *rock, *dirt;  // eroded rock and dirt
};

// ---- k2f_hydro ----------------------------------------------------------------
template <bool EDGE>
__device__ __forceinline__ void hydro_tile(const HydroArgs& a, float* sm, uint64_t* bar, int tx0, int ty0,
                                           int* err) {
    const StepConsts& c = a.c;
    const RainStep& r = a.r;
    const int n = c.n;
    const int tid = threadIdx.x;
    const int gx0 = tx0 - HX, gy0 = ty0 - 1;
    if (tid == 0) {
        mbar_arrive_expect_tx(bar, F_N * H_BOX * sizeof(float));
#pragma unroll
        for (int f = 0; f < F_N; ++f) tma_load_2d(sm + f * H_RC, &a.maps[f], gx0, gy0, bar);
    }
    constexpr int RG = (RW / 4) * H_RH;
    constexpr int RGK = (RG + NT - 1) / NT;
    uint32_t words[RGK][4];
#pragma unroll
    for (int k = 0; k < RGK; ++k) {
        words[k][0] = words[k][1] = words[k][2] = words[k][3] = 0;
        int q = tid + k * NT;
        if (q < RG && r.active && r.bernoulli) {
            int gx = gx0 + (q % (RW / 4)) * 4, gy = gy0 + q / (RW / 4);
            if (!EDGE || (gx >= 0 && gx < n && gy >= 0 && gy < n)) rain_words4(r, gx, gy, words[k]);
        }
    }
    bool ok = __syncthreads_and(mbar_wait(bar, 0));
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        mbar_wait(bar, 0);
        return;
    }
    if (r.active) {
        float* D = sm + F_D * H_RC;
#pragma unroll
        for (int k = 0; k < RGK; ++k) {
            int q = tid + k * NT;
            if (q >= RG) continue;
            int rx = (q % (RW / 4)) * 4, ry = q / (RW / 4);
            int gx = gx0 + rx, gy = gy0 + ry;
            if (EDGE && !(gx >= 0 && gx < n && gy >= 0 && gy < n)) continue;
            float4 d = ld4(D + ry * RW + rx);
            d.x += rain_incr(r, words[k][0]);
            d.y += rain_incr(r, words[k][1]);
            d.z += rain_incr(r, words[k][2]);
            d.w += rain_incr(r, words[k][3]);
            st4(D + ry * RW + rx, d);
        }
    }
    __syncthreads();
    const float* B = sm + F_B * H_RC;
    const float* G = sm + F_G * H_RC;
    const float* D = sm + F_D * H_RC;
    const float* S0 = sm + F_S0 * H_RC;
    const float* S1 = sm + F_S1 * H_RC;
    const float* FL = sm + F_FL * H_RC;
    const float* FR = sm + F_FR * H_RC;
    const float* FT = sm + F_FT * H_RC;
    const float* FB = sm + F_FB * H_RC;
#pragma unroll 1
    for (int k = 0; k < TW * TH / NT; ++k) {
        const int q = tid + k * NT;
        const int ix = q % TW, iy = q / TW;
        const int x = tx0 + ix, y = ty0 + iy;
        const int si = (1 + iy) * RW + HX + ix;
        const size_t gi = (size_t)y * n + x;
        const bool has_l = !EDGE || x > 0, has_r = !EDGE || x < n - 1;
        const bool has_b = !EDGE || y > 0, has_t = !EDGE || y < n - 1;
        float b = B[si], g = G[si], d1 = D[si];
        const float bl = B[si - 1], br = B[si + 1], bb = B[si - RW], bt = B[si + RW];
        const float gl = G[si - 1], gr = G[si + 1], gb = G[si - RW], gt = G[si + RW];
        // the two-layer total (rock + dirt) + water
        const float w_c = b + g + d1;
        const float wl = has_l ? bl + gl + D[si - 1] : FAR_HEIGHT;
        const float wr = has_r ? br + gr + D[si + 1] : FAR_HEIGHT;
        const float wt = has_t ? bt + gt + D[si + RW] : FAR_HEIGHT;
        const float wb = has_b ? bb + gb + D[si - RW] : FAR_HEIGHT;
        const float inl = has_l ? FR[si - 1] : 0.0f;
        const float inr = has_r ? FL[si + 1] : 0.0f;
        const float int_ = has_t ? FB[si + RW] : 0.0f;
        const float inb = has_b ? FT[si - RW] : 0.0f;
        FluxOut o = cell_flux(c, x, y, w_c, d1, FL[si], FR[si], FT[si], FB[si], wl, wr, wt, wb, inl, inr, int_, inb,
                              EDGE);
        float s0 = S0[si], s1 = S1[si];
        const float Kls0 = c.ks_field ? c.dt * __ldg(c.ks_field + gi) : c.Kls0;
        cell_erosion2(c, Kls0, o.u, o.v, o.vz, b, g, s0, s1, has_r ? br : 0.0f, has_r ? gr : 0.0f,
                      has_l ? bl : 0.0f, has_l ? gl : 0.0f, has_t ? bt : 0.0f, has_t ? gt : 0.0f,
                      has_b ? bb : 0.0f, has_b ? gb : 0.0f);
        a.fl[gi] = o.fl;
        a.fr[gi] = o.fr;
        a.ft[gi] = o.ft;
        a.fb[gi] = o.fb;
        a.water[gi] = o.d2 * c.evap;  // sediment_transport's evaporation
        a.u[gi] = o.u;
        a.v[gi] = o.v;
        a.s0[gi] = s0;
        a.s1[gi] = s1;
        a.rock[gi] = b;
        a.dirt[gi] = g;
    }
}

__global__ void __launch_bounds__(NT) k2f_hydro(const __grid_constant__ HydroArgs a, int* err) {
    __shared__ __align__(128) float sm[F_N * H_RC];
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    const int n = a.c.n;
    const int tiles_x = n / TW;
    const int tx0 = (blockIdx.x % tiles_x) * TW, ty0 = (blockIdx.x / tiles_x) * TH;
    const bool inner = tx0 - HX >= 0 && tx0 + TW + HX <= n && ty0 - 1 >= 0 && ty0 + TH + 1 <= n;
    if (inner) hydro_tile<false>(a, sm, &bar, tx0, ty0, err);
    else hydro_tile<true>(a, sm, &bar, tx0, ty0, err);
}

// ---- k2f_transport --------------------------------------------------------------
struct TransportArgs {
    CUtensorMap map_be;  // eroded rock, 72 x 20 boxes
    StepConsts c;
    int sediment;        // 0: the rock talus pass alone (particle mode)
    const float *u, *v, *s0, *s1;  // velocity, eroded sediment (rock, dirt)
    float *s0_o, *s1_o;            // transported sediment
    float* rock_o;                 // rock after the layer-0 talus pass
};

// eight rock-talus outflows of region cell (rx, ry), global (gx, gy); 0 outside the grid
template <bool EDGE>
__device__ __forceinline__ void outflows0(const StepConsts& c, const float* be, int rx, int ry, int gx, int gy,
                                          float o8[8]) {
    const int n = c.n;
    if (EDGE && (gx < 0 || gx >= n || gy < 0 || gy >= n)) {
#pragma unroll
        for (int d = 0; d < 8; ++d) o8[d] = 0.0f;
        return;
    }
    const int si = ry * RW + rx;
    float nb[8];
#pragma unroll
    for (int d = 0; d < 8; ++d) {
        bool out = false;
        if (EDGE) {
            int xx = gx + f2_ox[d], yy = gy + f2_oy[d];
            out = xx < 0 || xx >= n || yy < 0 || yy >= n;
        }
        nb[d] = out ? FAR_HEIGHT : be[si + f2_oy[d] * RW + f2_ox[d]];
    }
    cell_thermal_outflows(c, be[si], nb, o8);
}

template <bool EDGE>
__device__ __forceinline__ void transport_tile(const TransportArgs& a, float* be, float* outf, uint64_t* bar, int tx0,
                                               int ty0, int* err) {
    const StepConsts& c = a.c;
    const int n = c.n;
    const int tid = threadIdx.x;
    const int gx0 = tx0 - HX, gy0 = ty0 - 2;
    if (c.thermal && tid == 0) {
        mbar_arrive_expect_tx(bar, T_BOX * sizeof(float));
        tma_load_2d(be, &a.map_be, gx0, gy0, bar);
    }
    const int iy = tid / GPR, g = tid % GPR;
    const int x0 = tx0 + 4 * g, y = ty0 + iy;
    const size_t gi0 = (size_t)y * n + x0;
    float bx[4], by[4], ta[4][4], tb[4][4];
    if (a.sediment) {
    const float4 u4 = __ldg(reinterpret_cast<const float4*>(a.u + gi0));
    const float4 v4 = __ldg(reinterpret_cast<const float4*>(a.v + gi0));
    // sediment_transport, both channels: one back-trace, two gathers.  The
    // taps' loads stay in flight across the tile's TMA wait; the bilinear
    // mixes follow it (later, the talus registers would spill).
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        backtrace(c, x0 + j, y, at4(u4, j), at4(v4, j), bx[j], by[j]);
        const int ix = (int)bx[j], iy2 = (int)by[j];  // in [0, n - 1]
        const bool hx = ix + 1 < n, hy = iy2 + 1 < n;
        const size_t o = (size_t)iy2 * n + ix;
        const float* p0 = a.s0 + o;
        const float* p1 = a.s1 + o;
        ta[j][0] = __ldg(p0); ta[j][1] = hx ? __ldg(p0 + 1) : 0.0f;
        ta[j][2] = hy ? __ldg(p0 + n) : 0.0f; ta[j][3] = (hx && hy) ? __ldg(p0 + n + 1) : 0.0f;
        tb[j][0] = __ldg(p1); tb[j][1] = hx ? __ldg(p1 + 1) : 0.0f;
        tb[j][2] = hy ? __ldg(p1 + n) : 0.0f; tb[j][3] = (hx && hy) ? __ldg(p1 + n + 1) : 0.0f;
    }
    }
    auto finish_sed = [&]() {
        if (!a.sediment) return;
        float sa[4], sb[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            sa[j] = bilinear_mix(bx[j], by[j], ta[j][0], ta[j][1], ta[j][2], ta[j][3]);
            sb[j] = bilinear_mix(bx[j], by[j], tb[j][0], tb[j][1], tb[j][2], tb[j][3]);
        }
        st4(a.s0_o + gi0, make_float4(sa[0], sa[1], sa[2], sa[3]));
        st4(a.s1_o + gi0, make_float4(sb[0], sb[1], sb[2], sb[3]));
    };
    if (!c.thermal) {
        finish_sed();
        return;
    }

    bool ok = __syncthreads_and(mbar_wait(bar, 0));
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        mbar_wait(bar, 0);
        return;
    }
    finish_sed();
    // outflows of the interior (one row group per thread), own sums in registers
    const int rx0 = HX + 4 * g, ry = 2 + iy;
    const int oi = (ry - 1) * RW + rx0;
    float osum[4];
    {
        const int si = ry * RW + rx0;
        const float4 m4 = ld4(be + si - RW), c4 = ld4(be + si), p4 = ld4(be + si + RW);
        const float ml = be[si - RW - 1], mr = be[si - RW + 4];
        const float cl = be[si - 1], cr = be[si + 4];
        const float pl = be[si + RW - 1], pr = be[si + RW + 4];
        float o[8][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int x = x0 + j;
            const bool has_l = !EDGE || x > 0, has_r = !EDGE || x < n - 1;
            const bool has_b = !EDGE || y > 0, has_t = !EDGE || y < n - 1;
            float nb[8];
            nb[0] = has_l ? (j == 0 ? cl : at4(c4, j - 1)) : FAR_HEIGHT;
            nb[1] = has_r ? (j == 3 ? cr : at4(c4, j + 1)) : FAR_HEIGHT;
            nb[2] = has_t ? at4(p4, j) : FAR_HEIGHT;
            nb[3] = has_b ? at4(m4, j) : FAR_HEIGHT;
            nb[4] = (has_l && has_t) ? (j == 0 ? pl : at4(p4, j - 1)) : FAR_HEIGHT;
            nb[5] = (has_r && has_t) ? (j == 3 ? pr : at4(p4, j + 1)) : FAR_HEIGHT;
            nb[6] = (has_l && has_b) ? (j == 0 ? ml : at4(m4, j - 1)) : FAR_HEIGHT;
            nb[7] = (has_r && has_b) ? (j == 3 ? mr : at4(m4, j + 1)) : FAR_HEIGHT;
            float o8[8];
            cell_thermal_outflows(c, at4(c4, j), nb, o8);
            osum[j] = 0.0f;
#pragma unroll
            for (int d = 0; d < 8; ++d) {
                o[d][j] = o8[d];
                osum[j] -= o8[d];
            }
        }
#pragma unroll
        for (int d = 0; d < 8; ++d) st4(outf + d * O_C + oi, make_float4(o[d][0], o[d][1], o[d][2], o[d][3]));
    }
    // the ring of interior plus 1
    {
        constexpr int RING = 2 * TW + 2 * (TH + 2);
        for (int q = tid; q < RING; q += NT) {
            int rx, ry2;
            if (q < TW) { rx = HX + q; ry2 = 1; }
            else if (q < 2 * TW) { rx = HX + q - TW; ry2 = TH + 2; }
            else if (q < 2 * TW + TH + 2) { rx = HX - 1; ry2 = 1 + q - 2 * TW; }
            else { rx = HX + TW; ry2 = 1 + q - 2 * TW - (TH + 2); }
            float o8[8];
            outflows0<EDGE>(c, be, rx, ry2, gx0 + rx, gy0 + ry2, o8);
            const int ro = (ry2 - 1) * RW + rx;
#pragma unroll
            for (int d = 0; d < 8; ++d) outf[d * O_C + ro] = o8[d];
        }
    }
    __syncthreads();
    // thermal_transport: rock = b + (sum + inflow), inflows L.R, R.L, T.B, B.T, LT.RB, RT.LB, LB.RT, RB.LT
    {
        const unsigned FULL = 0xffffffffu;
        const bool first = g == 0, last = g == GPR - 1;
        const float4 oL = ld4(outf + 0 * O_C + oi), oR = ld4(outf + 1 * O_C + oi);
        float pR = __shfl_up_sync(FULL, oR.w, 1);
        float nL = __shfl_down_sync(FULL, oL.x, 1);
        if (first) pR = outf[1 * O_C + oi - 1];
        if (last) nL = outf[0 * O_C + oi + 4];
        float inf[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            inf[j] = 0.0f;
            inf[j] += j == 0 ? pR : at4(oR, j - 1);
            inf[j] += j == 3 ? nL : at4(oL, j + 1);
        }
        const float4 inT = ld4(outf + 3 * O_C + oi + RW);
        const float4 inB = ld4(outf + 2 * O_C + oi - RW);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            inf[j] += at4(inT, j);
            inf[j] += at4(inB, j);
        }
        const float4 rbT = ld4(outf + 7 * O_C + oi + RW), lbT = ld4(outf + 6 * O_C + oi + RW);
        float pRB = __shfl_up_sync(FULL, rbT.w, 1), nLB = __shfl_down_sync(FULL, lbT.x, 1);
        if (first) pRB = outf[7 * O_C + oi + RW - 1];
        if (last) nLB = outf[6 * O_C + oi + RW + 4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            inf[j] += j == 0 ? pRB : at4(rbT, j - 1);
            inf[j] += j == 3 ? nLB : at4(lbT, j + 1);
        }
        const float4 rtB = ld4(outf + 5 * O_C + oi - RW), ltB = ld4(outf + 4 * O_C + oi - RW);
        float pRT = __shfl_up_sync(FULL, rtB.w, 1), nLT = __shfl_down_sync(FULL, ltB.x, 1);
        if (first) pRT = outf[5 * O_C + oi - RW - 1];
        if (last) nLT = outf[4 * O_C + oi - RW + 4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            inf[j] += j == 0 ? pRT : at4(rtB, j - 1);
            inf[j] += j == 3 ? nLT : at4(ltB, j + 1);
        }
        const float4 b4 = ld4(be + ry * RW + rx0);
        float res[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) res[j] = at4(b4, j) + (osum[j] + inf[j]);
        st4(a.rock_o + gi0, make_float4(res[0], res[1], res[2], res[3]));
    }
}

__global__ void __launch_bounds__(NT, 4) k2f_transport(const __grid_constant__ TransportArgs a, int* err) {
    __shared__ __align__(128) float be[T_BOX];
    __shared__ __align__(16) float outf[8 * O_C];
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    const int n = a.c.n;
    const int tiles_x = n / TW;
    const int tx0 = (blockIdx.x % tiles_x) * TW, ty0 = (blockIdx.x / tiles_x) * TH;
    const bool inner = tx0 - HX >= 0 && tx0 + TW + HX <= n && ty0 - 2 >= 0 && ty0 + TH + 2 <= n;
    if (inner) transport_tile<false>(a, be, outf, &bar, tx0, ty0, err);
    else transport_tile<true>(a, be, outf, &bar, tx0, ty0, err);
}

// ---- k2f_layer1 -----------------------------------------------------------------
struct Layer1Args {
    CUtensorMap map_r, map_g;  // rock after layer 0, dirt after erosion: 72 x 22 boxes
    StepConsts c;
    Talus1 t1;
    int thermal1;              // layer-1 talus pass on (Kspeed[1] != 0)
    float *rock_o, *dirt_o;
    // particle mode: smoothing's particle branch (glsl/smoothing.glsl:76-95),
    // per cell: momentum fold and water decay
    int particle;
    float count;               // droplets
    const float* water;
    float* water_o;
    const float* mom[4];
    float* mom_o[4];
};

// region (rx, ry) of the staged boxes <-> global (tx0 - HX + rx, ty0 - 3 + ry);
// outflow planes cover rx in [2, 70), ry in [1, 21): plane index (ry - 1) * P_W + rx - 2
template <bool EDGE>
__device__ __forceinline__ void layer1_tile(const Layer1Args& a, float* R, float* Gd, float* P, uint64_t* bar, int tx0,
                                            int ty0, int* err) {
    const StepConsts& c = a.c;
    const int n = c.n;
    const int tid = threadIdx.x;
    const int gx0 = tx0 - HX, gy0 = ty0 - 3;
    if (tid == 0) {
        mbar_arrive_expect_tx(bar, 2 * L_BOX * sizeof(float));
        tma_load_2d(R, &a.map_r, gx0, gy0, bar);
        tma_load_2d(Gd, &a.map_g, gx0, gy0, bar);
    }
    bool ok = __syncthreads_and(mbar_wait(bar, 0));
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        mbar_wait(bar, 0);
        return;
    }
    auto inside = [&](int gx, int gy) { return !EDGE || (gx >= 0 && gx < n && gy >= 0 && gy < n); };
    if (a.thermal1) {
        // outflows of the tile plus two rings (0 outside the grid)
        for (int q = tid; q < P_C; q += NT) {
            const int px = q % P_W, py = q / P_W;
            const int rx = px + 2, ry = py + 1;
            const int gx = gx0 + rx, gy = gy0 + ry;
            float o8[8];
            if (!inside(gx, gy)) {
#pragma unroll
                for (int d = 0; d < 8; ++d) o8[d] = 0.0f;
            } else {
                const int si = ry * RW + rx;
                const float r = R[si], gg = Gd[si];
                float dh[8];
#pragma unroll
                for (int d = 0; d < 8; ++d) {
                    const bool in = inside(gx + f2_ox[d], gy + f2_oy[d]);
                    const int sj = si + f2_oy[d] * RW + f2_ox[d];
                    const float nr = in ? R[sj] : FAR_HEIGHT, ng = in ? Gd[sj] : FAR_HEIGHT;
                    dh[d] = (0.0f + (r - nr)) + (gg - ng);
                }
                cell_thermal_outflows1(c, a.t1, dh, gg, o8);
            }
#pragma unroll
            for (int d = 0; d < 8; ++d) P[d * P_C + q] = o8[d];
        }
        __syncthreads();
        // dirt transport on the tile plus one ring, in place in the dirt box
        // (cells outside the grid keep their 0)
        constexpr int TR_W = TW + 2, TR_H = TH + 2;
        float res[(TR_W * TR_H + NT - 1) / NT];
#pragma unroll
        for (int k = 0; k < (TR_W * TR_H + NT - 1) / NT; ++k) {
            const int q = tid + k * NT;
            res[k] = 0.0f;
            if (q >= TR_W * TR_H) continue;
            const int rx = HX - 1 + q % TR_W, ry = 2 + q / TR_W;
            const int gx = gx0 + rx, gy = gy0 + ry;
            if (!inside(gx, gy)) continue;
            const int pi = (ry - 1) * P_W + rx - 2;
            float own[8], in[8];
#pragma unroll
            for (int d = 0; d < 8; ++d) own[d] = P[d * P_C + pi];
            in[0] = P[1 * P_C + pi - 1];            // L neighbour's R
            in[1] = P[0 * P_C + pi + 1];            // R neighbour's L
            in[2] = P[3 * P_C + pi + P_W];          // T neighbour's B
            in[3] = P[2 * P_C + pi - P_W];          // B neighbour's T
            in[4] = P[7 * P_C + pi + P_W - 1];      // LT neighbour's RB
            in[5] = P[6 * P_C + pi + P_W + 1];      // RT neighbour's LB
            in[6] = P[5 * P_C + pi - P_W - 1];      // LB neighbour's RT
            in[7] = P[4 * P_C + pi - P_W + 1];      // RB neighbour's LT
            res[k] = cell_thermal_apply(Gd[ry * RW + rx], own, in);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < (TR_W * TR_H + NT - 1) / NT; ++k) {
            const int q = tid + k * NT;
            if (q >= TR_W * TR_H) continue;
            const int rx = HX - 1 + q % TR_W, ry = 2 + q / TR_W;
            if (!inside(gx0 + rx, gy0 + ry)) continue;
            Gd[ry * RW + rx] = res[k];
        }
        __syncthreads();
    }
    // smoothing of the tile (border texels of the grid are copied)
#pragma unroll 1
    for (int k = 0; k < TW * TH / NT; ++k) {
        const int q = tid + k * NT;
        const int ix = q % TW, iy = q / TW;
        const int x = tx0 + ix, y = ty0 + iy;
        const int si = (3 + iy) * RW + HX + ix;
        float r = R[si], gg = Gd[si];
        const bool border = x == 0 || y == 0 || x == n - 1 || y == n - 1;
        const size_t gi = (size_t)y * n + x;
        if (a.particle) {
            // border texels copy their heights and water and leave the
            // momentum map's write buffer as it was
            float wat = a.water[gi];
            if (!border) {
                cell_smooth2(c.smooth_m, r, gg, R[si - 1], Gd[si - 1], R[si + 1], Gd[si + 1], R[si + RW],
                             Gd[si + RW], R[si - RW], Gd[si - RW]);
                float mx = a.mom[0][gi], my = a.mom[1][gi], mz = a.mom[2][gi], mw = a.mom[3][gi];
                const float keep = gclamp(1.0f - 1e-12f * a.count, 0.0f, 1.0f);
                mx *= keep;
                my *= keep;
                mx += 1e-12f * a.count * mz;
                my += 1e-12f * a.count * mw;
                wat *= gclamp(1.0f - 8e-8f * a.count, 0.0f, 1.0f);
                if (wat < 1e-6f) wat = 0.0f;
                if (sqrtf(mx * mx + my * my) < 1e-12f) {
                    mx = 0.0f;
                    my = 0.0f;
                }
                a.mom_o[0][gi] = mx;
                a.mom_o[1][gi] = my;
                a.mom_o[2][gi] = 0.0f;
                a.mom_o[3][gi] = 0.0f;
            }
            a.water_o[gi] = wat;
        } else if (c.smooth_m != 0.0f && !border) {
            cell_smooth2(c.smooth_m, r, gg, R[si - 1], Gd[si - 1], R[si + 1], Gd[si + 1], R[si + RW], Gd[si + RW],
                         R[si - RW], Gd[si - RW]);
        }
        a.rock_o[gi] = r;
        a.dirt_o[gi] = gg;
    }
}

constexpr size_t LAYER1_SMEM = (2 * L_RC + 8 * P_C) * sizeof(float) + 16;

__global__ void __launch_bounds__(NT) k2f_layer1(const __grid_constant__ Layer1Args a, int* err) {
    extern __shared__ __align__(128) float dyn[];
    float* R = dyn;
    float* Gd = dyn + L_RC;
    float* P = dyn + 2 * L_RC;
    uint64_t* bar = reinterpret_cast<uint64_t*>(dyn + 2 * L_RC + 8 * P_C);
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    const int n = a.c.n;
    const int tiles_x = n / TW;
    const int tx0 = (blockIdx.x % tiles_x) * TW, ty0 = (blockIdx.x / tiles_x) * TH;
    const bool inner = tx0 - HX >= 0 && tx0 + TW + HX <= n && ty0 - 3 >= 0 && ty0 + TH + 3 <= n;
    if (inner) layer1_tile<false>(a, R, Gd, P, bar, tx0, ty0, err);
    else layer1_tile<true>(a, R, Gd, P, bar, tx0, ty0, err);
}

}  // namespace

bool fused2_ok(int n) { return n % TW == 0 && n % TH == 0; }

int launch_fused2_step(const StepConsts& c, const Talus1& t1, const RainStep& r, const Fused2Bufs& b, TmaCache& tma,
                       int* err, cudaStream_t st) {
    const int n = c.n;
    const int tiles = (n / TW) * (n / TH);
    const bool l0 = c.thermal != 0;
    const bool l1 = c.Kspeed1 != 0.0f || c.smooth_m != 0.0f;  // k2f_layer1 runs
    // where each stage leaves rock and dirt
    float* rock_eroded = l0 ? b.b_ero : (l1 ? b.rock_mid : b.rock_o);
    float* rock_l0 = l1 ? b.rock_mid : b.rock_o;
    float* dirt_eroded = l1 ? b.g_ero : b.dirt_o;

    HydroArgs ha{};
    const float* ins[F_N] = {b.rock, b.dirt, b.water, b.s0, b.s1, b.fl, b.fr, b.ft, b.fb};
    for (int f = 0; f < F_N; ++f)
        if (!tma.get(ins[f], n, H_RH, &ha.maps[f])) return HG_ERR_CUDA;
    ha.c = c;
    ha.r = r;
    ha.water = b.water_o; ha.fl = b.fl_o; ha.fr = b.fr_o; ha.ft = b.ft_o; ha.fb = b.fb_o;
    ha.u = b.u; ha.v = b.v;
    ha.s0 = b.s0_ero; ha.s1 = b.s1_ero;
    ha.rock = rock_eroded;
    ha.dirt = dirt_eroded;
    k2f_hydro<<<tiles, NT, 0, st>>>(ha, err);

    TransportArgs ta{};
    if (l0 && !tma.get(b.b_ero, n, T_RH, &ta.map_be)) return HG_ERR_CUDA;
    ta.c = c;
    ta.sediment = 1;
    ta.u = b.u; ta.v = b.v;
    ta.s0 = b.s0_ero; ta.s1 = b.s1_ero;
    ta.s0_o = b.s0_o; ta.s1_o = b.s1_o;
    ta.rock_o = rock_l0;
    k2f_transport<<<tiles, NT, 0, st>>>(ta, err);
    count_launch(2);

    if (l1) {
        Layer1Args la{};
        if (!tma.get(rock_l0, n, L_RH, &la.map_r) || !tma.get(dirt_eroded, n, L_RH, &la.map_g)) return HG_ERR_CUDA;
        la.c = c;
        la.t1 = t1;
        la.thermal1 = c.Kspeed1 != 0.0f ? 1 : 0;
        la.rock_o = b.rock_o;
        la.dirt_o = b.dirt_o;
        // per device and cheap: set on every launch rather than cached
        cudaFuncSetAttribute(k2f_layer1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LAYER1_SMEM);
        k2f_layer1<<<tiles, NT, LAYER1_SMEM, st>>>(la, err);
        count_launch();
    }
    return HG_OK;
}

int launch_particle_thermal_smooth(const StepConsts& c, const Talus1& t1, float count, const PWorld& in,
                                   const PWorld& out, float* rock_mid, TmaCache& tma, int* err, cudaStream_t st) {
    const int n = c.n;
    const int tiles = (n / TW) * (n / TH);
    const float* rock_l0 = in.rock;
    if (c.thermal) {  // the rock talus pass alone
        TransportArgs ta{};
        if (!tma.get(in.rock, n, T_RH, &ta.map_be)) return HG_ERR_CUDA;
        ta.c = c;
        ta.sediment = 0;
        ta.rock_o = rock_mid;
        k2f_transport<<<tiles, NT, 0, st>>>(ta, err);
        count_launch();
        rock_l0 = rock_mid;
    }
    Layer1Args la{};
    if (!tma.get(rock_l0, n, L_RH, &la.map_r) || !tma.get(in.dirt, n, L_RH, &la.map_g)) return HG_ERR_CUDA;
    la.c = c;
    la.t1 = t1;
    la.thermal1 = c.Kspeed1 != 0.0f ? 1 : 0;
    la.rock_o = out.rock;
    la.dirt_o = out.dirt;
    la.particle = 1;
    la.count = count;
    la.water = in.water;
    la.water_o = out.water;
    for (int k = 0; k < 4; ++k) {
        la.mom[k] = in.mom[k];
        la.mom_o[k] = out.mom[k];
    }
    cudaFuncSetAttribute(k2f_layer1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LAYER1_SMEM);
    k2f_layer1<<<tiles, NT, LAYER1_SMEM, st>>>(la, err);
    count_launch();
    return HG_OK;
}

}  // namespace hg
