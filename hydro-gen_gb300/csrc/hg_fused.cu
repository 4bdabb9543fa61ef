// Fused grid step in two kernels:
//   k_hydro:      rain -> hydro_flux -> hydro_erosion (+ evaporation)
//   k_transport:  sediment_transport -> thermal_erosion/thermal_transport
// replacing the reference's six dispatches per step (src/erosion.cpp:158-200).
//
// Why two and not one: every pass of k_hydro needs only its neighbours'
// INPUTS (rock, water, flux), so it runs with no redundant work; the passes
// of k_transport need neighbours' RESULTS of k_hydro (eroded rock for the
// talus test, eroded sediment for the back-trace).  The sediment back-trace
// reach |u|*dt is unbounded (velocity divides by the water depth, and thin
// films give reaches of thousands of cells), so no halo can hold it; after
// k_hydro has written the eroded sediment of every cell, k_transport gathers
// any tap straight from L2/HBM.  The split costs 16 B per cell-step of
// intermediate traffic (eroded rock and sediment written and read once) and
// saves recomputing flux and erosion on a halo ring.
//
// Both kernels are table driven: one launch covers every tile of any number
// of worlds ("terrains") of different sizes and settings.  A block finds its
// terrain by binary search over the terrains' first tile (k_hydro) or first
// block (k_transport) and reads the terrain's record (step constants, rain
// settings, buffers, step counter; TMA tensor maps in global memory).  A
// single world takes its whole descriptor, tensor maps included, as a kernel
// parameter.  The rain step number comes from the terrain's device step
// counter (advanced by k_transport), so a captured CUDA graph of a few steps
// can be replayed any number of times.
//
//   k_hydro stages rock, water, sediment and the four fluxes of a 64 x TH
//   tile plus a halo (4 columns, 1 row) with seven TMA 2-D tile loads; while
//   they fly, threads draw this step's Philox rain words; rain is then added
//   in shared memory.  Each thread computes TW*TH/NTH cells, one per
//   iteration (low register use keeps ~6 blocks per SM to hide the long
//   dependent chains of flux and erosion), a warp covering 32 consecutive
//   cells of a row.
//   k_transport: see its section below (talus warps sweeping a run of tiles
//   with TMA double buffering, gather warps beside them).
//
// Per-cell arithmetic is the code of the per-pass kernels (hg_device.cuh),
// evaluated two cells per f32x2 instruction where cells pair up, so the
// fused step reproduces the per-pass kernels bit for bit.
#include <cudaTypedefs.h>

#include <mutex>
#include <vector>

#include "hg_internal.h"
#include "hg_tma.cuh"

namespace hg {

namespace {

constexpr int TW = 64;
constexpr int GPR = TW / 4;      // row groups per tile row (16)
constexpr int HX = 4;            // halo columns: 16-byte aligned TMA boxes
constexpr int RW = TW + 2 * HX;  // 72
enum { H_B = 0, H_D, H_S, H_FL, H_FR, H_FT, H_FB, H_N };
constexpr int M_BERO = H_N;      // tensor map index of the eroded rock

// Geometry of a 64 x TH tile: TH = 16 with 256 threads or TH = 8 with 128.
template <int TH>
struct Geo {
    static constexpr int NTH = TH * GPR;                 // k_hydro: 4 cells per thread
    static constexpr int H_RH = TH + 2, H_BOX = RW * H_RH;
    static constexpr int H_RC = ((H_BOX + 31) / 32) * 32;  // 128-byte aligned array stride
    static constexpr int T_RH = TH + 4, T_BOX = RW * T_RH;
    static constexpr int CPT = TW * TH / NTH;             // cells per thread in k_hydro (4)
};

// direction d: L, R, T, B, LT, RT, LB, RB
__constant__ int f_ox[8] = {-1, 1, 0, 0, -1, 1, -1, 1};
__constant__ int f_oy[8] = {0, 0, 1, -1, 1, 1, -1, -1};

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float at4(const float4& v, int j) { return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w; }

__device__ __forceinline__ int find_terrain(const int* tile0, int nterr, int tile) {
    int lo = 0, hi = nterr - 1;
    while (lo < hi) {  // last terrain whose first tile <= tile
        int mid = (lo + hi + 1) >> 1;
        if (tile0[mid] <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ RainStep rain_for(const RainBase& rb, unsigned long long step1) {
    RainStep r;
    // uniform and Bernoulli rain only: the reference rain runs as its own
    // kernel before the step (the host inserts it)
    r.active = ((rb.mode == 1 || rb.mode == 2) && rb.period > 0 && step1 % (unsigned long long)rb.period == 0ull) ? 1 : 0;
    r.bernoulli = rb.mode == 2 ? 1 : 0;
    r.amount = rb.amount;
    r.threshold = rb.threshold;
    r.seed_lo = rb.seed_lo;
    r.seed_hi = rb.seed_hi;
    r.terrain_id = rb.terrain_id;
    r.step = (uint32_t)step1;
    return r;
}

// ---------------------------------------------------------------------------
// k_hydro
// ---------------------------------------------------------------------------
template <int TH, bool EDGE>
__device__ __forceinline__ void hydro_tile(const TerrainHot& td, const CUtensorMap* maps, float* sm, uint64_t* bar,
                                           int tx0, int ty0, int* err) {
    using G = Geo<TH>;
    constexpr int NTH = G::NTH, H_RC = G::H_RC, H_RH = G::H_RH;
    const StepConsts& c = td.c;
    const int n = c.n;
    const int tid = threadIdx.x;
    const int gx0 = tx0 - HX, gy0 = ty0 - 1;
    if (tid == 0) {
        mbar_arrive_expect_tx(bar, H_N * G::H_BOX * sizeof(float));
#pragma unroll
        for (int f = 0; f < H_N; ++f) tma_load_2d(sm + f * H_RC, &maps[f], gx0, gy0, bar);
    }
    // the step counter's load overlaps the tiles' copies
    const RainStep r = rain_for(td.rain, *td.step + 1ull);
    // rain words of the region's row groups, drawn while the tiles load
    constexpr int RG = (RW / 4) * H_RH;
    constexpr int RGK = (RG + NTH - 1) / NTH;
    uint32_t words[RGK][4];
#pragma unroll
    for (int k = 0; k < RGK; ++k) {
        words[k][0] = words[k][1] = words[k][2] = words[k][3] = 0;
        int q = tid + k * NTH;
        if (q < RG && r.active && r.bernoulli) {
            int gx = gx0 + (q % (RW / 4)) * 4, gy = gy0 + q / (RW / 4);
            if (!EDGE || (gx >= 0 && gx < n && gy >= 0 && gy < n)) rain_words4(r, gx, gy, words[k]);
        }
    }
    bool ok = __syncthreads_and(mbar_wait(bar, 0));
    if (!ok) {  // the tile never arrived: record, give the copies one more bounded wait, skip the tile
        if (tid == 0) atomicExch(err, 1);
        mbar_wait(bar, 0);
        return;
    }
    if (r.active) {
        float* D = sm + H_D * H_RC;
#pragma unroll
        for (int k = 0; k < RGK; ++k) {
            int q = tid + k * NTH;
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

    const float* B = sm + H_B * H_RC;
    const float* D = sm + H_D * H_RC;
    const float* S = sm + H_S * H_RC;
    const float* FL = sm + H_FL * H_RC;
    const float* FR = sm + H_FR * H_RC;
    const float* FT = sm + H_FT * H_RC;
    const float* FB = sm + H_FB * H_RC;
#pragma unroll 1
    for (int k = 0; k < G::CPT; ++k) {
        const int q = tid + k * NTH;
        const int ix = q % TW, iy = q / TW;
        const int x = tx0 + ix, y = ty0 + iy;
        const int si = (1 + iy) * RW + HX + ix;
        const size_t gi = (size_t)y * n + x;
        const bool has_l = !EDGE || x > 0, has_r = !EDGE || x < n - 1;
        const bool has_b = !EDGE || y > 0, has_t = !EDGE || y < n - 1;
        float b = B[si], d1 = D[si];
        float bl = B[si - 1], br = B[si + 1], bb = B[si - RW], bt = B[si + RW];
        float w_c = b + d1;
        float wl = has_l ? bl + D[si - 1] : FAR_HEIGHT;
        float wr = has_r ? br + D[si + 1] : FAR_HEIGHT;
        float wt = has_t ? bt + D[si + RW] : FAR_HEIGHT;
        float wb = has_b ? bb + D[si - RW] : FAR_HEIGHT;
        float inl = has_l ? FR[si - 1] : 0.0f;
        float inr = has_r ? FL[si + 1] : 0.0f;
        float int_ = has_t ? FB[si + RW] : 0.0f;
        float inb = has_b ? FT[si - RW] : 0.0f;
        FluxOut o = cell_flux(c, x, y, w_c, d1, FL[si], FR[si], FT[si], FB[si], wl, wr, wt, wb, inl, inr, int_, inb,
                              EDGE);
        float s = S[si];
        float Kls0 = c.ks_field ? c.dt * __ldg(c.ks_field + gi) : c.Kls0;
        cell_erosion(c, Kls0, o.u, o.v, o.vz, b, s, has_r ? br : 0.0f, has_l ? bl : 0.0f, has_b ? bb : 0.0f,
                     has_t ? bt : 0.0f);
        td.out[S_FL][gi] = o.fl;
        td.out[S_FR][gi] = o.fr;
        td.out[S_FT][gi] = o.ft;
        td.out[S_FB][gi] = o.fb;
        td.out[S_WATER][gi] = o.d2 * c.evap;  // sediment_transport's evaporation (glsl/sediment_transport.glsl:75)
        td.u[gi] = o.u;
        td.v[gi] = o.v;
        td.s_ero[gi] = s;
        (c.thermal ? td.b_ero : td.out[S_ROCK])[gi] = b;  // no thermal pass: eroded rock is final
    }
}

template <int TH>
__device__ __forceinline__ void hydro_block(const TerrainHot& td, const CUtensorMap* maps, int tile, int* err) {
    using G = Geo<TH>;
    __shared__ __align__(128) float sm[H_N * G::H_RC];
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    const int n = td.c.n;
    const int tx0 = (tile % td.tiles_x) * TW, ty0 = (tile / td.tiles_x) * TH;
    bool inner = tx0 - HX >= 0 && tx0 + TW + HX <= n && ty0 - 1 >= 0 && ty0 + TH + 1 <= n;
    if (inner) hydro_tile<TH, false>(td, maps, sm, &bar, tx0, ty0, err);
    else hydro_tile<TH, true>(td, maps, sm, &bar, tx0, ty0, err);
}

// Batch form: the terrain records are a kernel parameter (constant bank),
// the block finds its terrain by binary search.
template <int TH>
__global__ void __launch_bounds__(Geo<TH>::NTH) k_hydro(const __grid_constant__ BatchParams bp,
                                                        const CUtensorMap* __restrict__ maps, int* err) {
    const int t = find_terrain(bp.tile0, bp.nterr, blockIdx.x);
    hydro_block<TH>(bp.t[t], maps + MAPS_PER_TERRAIN * t, blockIdx.x - bp.tile0[t], err);
}

// Single-world form: the whole descriptor, tensor maps included, is a kernel
// parameter.
template <int TH>
__global__ void __launch_bounds__(Geo<TH>::NTH) k_hydro1(const __grid_constant__ TerrainDesc td, int* err) {
    hydro_block<TH>(td.h, td.maps, blockIdx.x, err);
}

// ---------------------------------------------------------------------------
// k_transport: sediment_transport and thermal_erosion/thermal_transport
// (layer 0), one block per vertical run of SEG tiles of one 64-column strip,
// with two kinds of warps:
//
//   talus warps sweep the run bottom to top.  The eroded rock of the next
//   tile is on its way by TMA (two stage buffers, one mbarrier each) while a
//   tile is computed.  Per tile they compute the talus outflows of the rows
//   ty0 + 1 .. ty0 + TH (all 66 columns: the tile's and the two columns
//   beside it) into shared memory, two cells per thread and f32x2 pair, and
//   then apply every cell's own outflows and its eight neighbours'
//   inflows.  Rows ty0 - 1 and ty0 were computed with the tile below and
//   stay in shared memory, so each row's outflows are computed once per run
//   instead of once per tile plus a two-row ring.  The work divides evenly:
//   TH x 33 pairs over the talus threads.
//
//   gather warps do the semi-Lagrangian sediment gather of the run's cells
//   from L2/HBM at their own pace (no barrier with the talus warps), so its
//   load latency overlaps the talus arithmetic.
// ---------------------------------------------------------------------------
template <int TH>
struct TGeo {
    static constexpr int TWP = TH == 16 ? 9 : 5;          // talus warps
    static constexpr int GWP = TH == 16 ? 4 : 2;          // gather warps
    static constexpr int TT = 32 * TWP;                   // talus threads
    static constexpr int GT = 32 * GWP;                   // gather threads
    static constexpr int NT = TT + GT;
    static constexpr int OR = TH + 2;                     // outflow rows held: ty0 - 1 .. ty0 + TH
    static constexpr int OPL = RW * OR;                   // outflow plane stride
    static constexpr int PLANES = 9;                      // eight directions + the own-outflow sum
    static constexpr int PPR = TW / 2 + 1;                // pairs per outflow row: 32 + the two side columns
    static constexpr int SEG = 8;                         // tiles per block
    static constexpr size_t SMEM = (2 * (size_t)Geo<TH>::T_BOX + PLANES * (size_t)OPL) * sizeof(float);
};

// Named barrier 1 over the talus warps only (the gather warps never join it).
template <int TH>
__device__ __forceinline__ void talus_sync() {
    asm volatile("bar.sync 1, %0;" ::"r"(TGeo<TH>::TT) : "memory");
}
template <int TH>
__device__ __forceinline__ bool talus_sync_and(bool p) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred pi, po;\n\t"
        "setp.ne.u32 pi, %1, 0;\n\t"
        "bar.red.and.pred po, 1, %2, pi;\n\t"
        "selp.u32 %0, 1, 0, po;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)p), "r"(TGeo<TH>::TT)
        : "memory");
    return r != 0;
}

// Talus outflows of a pair of cells from the staged eroded rock `be` (row 0
// = global row gy0): lanes .x and .y at region (rxa, rya) and (rxb, ryb).
// Neighbours outside the grid read FAR_HEIGHT; a cell outside the grid has
// no outflows.
template <bool EDGE>
__device__ __forceinline__ void pair_outflows(const StepConsts& c, const float* be, int rxa, int rya, int rxb,
                                              int ryb, int gx0, int gy0, float2 o[8]) {
    const int n = c.n;
    const int gxa = gx0 + rxa, gya = gy0 + rya, gxb = gx0 + rxb, gyb = gy0 + ryb;
    float2 nb[8];
#pragma unroll
    for (int d = 0; d < 8; ++d) {
        float va = be[(rya + f_oy[d]) * RW + rxa + f_ox[d]];
        float vb = be[(ryb + f_oy[d]) * RW + rxb + f_ox[d]];
        if (EDGE) {
            const int xa = gxa + f_ox[d], ya = gya + f_oy[d], xb = gxb + f_ox[d], yb = gyb + f_oy[d];
            if (xa < 0 || xa >= n || ya < 0 || ya >= n) va = FAR_HEIGHT;
            if (xb < 0 || xb >= n || yb < 0 || yb >= n) vb = FAR_HEIGHT;
        }
        nb[d] = make_float2(va, vb);
    }
    cell_thermal_outflows2(c, make_float2(be[rya * RW + rxa], be[ryb * RW + rxb]), nb, o);
    if (EDGE) {
        const bool ina = gxa >= 0 && gxa < n && gya >= 0 && gya < n;
        const bool inb = gxb >= 0 && gxb < n && gyb >= 0 && gyb < n;
#pragma unroll
        for (int d = 0; d < 8; ++d) {
            if (!ina) o[d].x = 0.0f;
            if (!inb) o[d].y = 0.0f;
        }
    }
}

// Outflow rows [r0, OR) of the tile at (tx0, ty0): outflow row lr is global
// row ty0 - 1 + lr, eroded-rock row lr + 1.  Pair k < 32 of a row is the
// cells tx0 + 2k, tx0 + 2k + 1; pair 32 the two side columns tx0 - 1 and
// tx0 + 64.  Each pair's eight outflows and the sums 0 - o[0] - ... - o[7]
// go to the planes.
template <int TH, bool EDGE>
__device__ __forceinline__ void talus_rows(const StepConsts& c, const float* be, float* outf, int tx0, int ty0,
                                           int r0, int tt) {
    using T = TGeo<TH>;
    const int npairs = (T::OR - r0) * T::PPR;
    const int gx0 = tx0 - HX, gy0 = ty0 - 2;
    for (int p = tt; p < npairs; p += T::TT) {
        const int lr = r0 + p / T::PPR, k = p % T::PPR;
        const bool side = k == T::PPR - 1;
        const int rxa = side ? HX - 1 : HX + 2 * k, rxb = side ? HX + TW : rxa + 1;
        float2 o[8];
        pair_outflows<EDGE>(c, be, rxa, lr + 1, rxb, lr + 1, gx0, gy0, o);
        float2 sum = pf(0.0f);
#pragma unroll
        for (int d = 0; d < 8; ++d) sum = sub2(sum, o[d]);
        const int oa = lr * RW + rxa, ob = lr * RW + rxb;
        if (!side) {  // adjacent and 8-byte aligned
#pragma unroll
            for (int d = 0; d < 8; ++d) *reinterpret_cast<float2*>(outf + d * T::OPL + oa) = o[d];
            *reinterpret_cast<float2*>(outf + 8 * T::OPL + oa) = sum;
        } else {
#pragma unroll
            for (int d = 0; d < 8; ++d) {
                outf[d * T::OPL + oa] = o[d].x;
                outf[d * T::OPL + ob] = o[d].y;
            }
            outf[8 * T::OPL + oa] = sum.x;
            outf[8 * T::OPL + ob] = sum.y;
        }
    }
}

// thermal_transport of the tile's row groups (four cells each): rock = b +
// (own sum + in_flux), in_flux = in[0] + ... + in[7] from 0 in the order L.R,
// R.L, T.B, B.T, LT.RB, RT.LB, LB.RT, RB.LT (cell_thermal_apply's operations).
template <int TH>
__device__ __forceinline__ void talus_apply(const TerrainHot& td, const float* be, const float* outf, int tx0,
                                            int ty0, int tt) {
    using T = TGeo<TH>;
    const int n = td.c.n;
    for (int q = tt; q < TH * GPR; q += T::TT) {
        const int iy = q / GPR, g = q % GPR;
        const int rx0 = HX + 4 * g;
        const int oi = (iy + 1) * RW + rx0;  // outflow row of global row ty0 + iy
        // left neighbour's direction-dl outflow and right neighbour's
        // direction-dr outflow, row at offset `off`, for the four cells
        auto row_in = [&](int dl, int dr, int off, float2 in[2][2]) {
            const float4 a = ld4(outf + dl * T::OPL + oi + off), b = ld4(outf + dr * T::OPL + oi + off);
            const float pa = outf[dl * T::OPL + oi + off - 1], nb = outf[dr * T::OPL + oi + off + 4];
            in[0][0] = make_float2(pa, a.x);
            in[0][1] = make_float2(a.y, a.z);
            in[1][0] = make_float2(b.y, b.z);
            in[1][1] = make_float2(b.w, nb);
        };
        float2 inf[2] = {pf(0.0f), pf(0.0f)};
        {
            float2 in[2][2];
            row_in(1, 0, 0, in);  // L neighbour's R, R neighbour's L
            inf[0] = add2(inf[0], in[0][0]); inf[1] = add2(inf[1], in[0][1]);
            inf[0] = add2(inf[0], in[1][0]); inf[1] = add2(inf[1], in[1][1]);
        }
        {
            const float4 inT = ld4(outf + 3 * T::OPL + oi + RW);  // top neighbour's B
            const float4 inB = ld4(outf + 2 * T::OPL + oi - RW);  // bottom neighbour's T
            inf[0] = add2(inf[0], make_float2(inT.x, inT.y)); inf[1] = add2(inf[1], make_float2(inT.z, inT.w));
            inf[0] = add2(inf[0], make_float2(inB.x, inB.y)); inf[1] = add2(inf[1], make_float2(inB.z, inB.w));
        }
        {
            float2 in[2][2];
            row_in(7, 6, RW, in);  // row above: LT neighbour's RB, RT neighbour's LB
            inf[0] = add2(inf[0], in[0][0]); inf[1] = add2(inf[1], in[0][1]);
            inf[0] = add2(inf[0], in[1][0]); inf[1] = add2(inf[1], in[1][1]);
        }
        {
            float2 in[2][2];
            row_in(5, 4, -RW, in);  // row below: LB neighbour's RT, RB neighbour's LT
            inf[0] = add2(inf[0], in[0][0]); inf[1] = add2(inf[1], in[0][1]);
            inf[0] = add2(inf[0], in[1][0]); inf[1] = add2(inf[1], in[1][1]);
        }
        const float4 own = ld4(outf + 8 * T::OPL + oi);
        const float4 b4 = ld4(be + (iy + 2) * RW + rx0);
        const float2 r0 = add2(make_float2(b4.x, b4.y), add2(make_float2(own.x, own.y), inf[0]));
        const float2 r1 = add2(make_float2(b4.z, b4.w), add2(make_float2(own.z, own.w), inf[1]));
        const size_t gi0 = (size_t)(ty0 + iy) * n + tx0 + 4 * g;
        st4(td.out[S_ROCK] + gi0, make_float4(r0.x, r0.y, r1.x, r1.y));
    }
}

// The semi-Lagrangian gather of the row group of four cells at (x0, y), as
// two pairs (glsl/sediment_transport.glsl:70-72, img_interpolation.glsl:3-22).
__device__ __forceinline__ void gather_group(const TerrainHot& td, int x0, int y) {
    const StepConsts& c = td.c;
    const int n = c.n;
    const size_t gi0 = (size_t)y * n + x0;
    const float4 u4 = __ldg(reinterpret_cast<const float4*>(td.u + gi0));
    const float4 v4 = __ldg(reinterpret_cast<const float4*>(td.v + gi0));
    float2 sed[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        float2 bx, by;
        backtrace2(c, x0 + 2 * h, y, make_float2(at4(u4, 2 * h), at4(u4, 2 * h + 1)),
                   make_float2(at4(v4, 2 * h), at4(v4, 2 * h + 1)), bx, by);
        float tap[4][2];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            const float px = l ? bx.y : bx.x, py = l ? by.y : by.x;
            const int ix = min(max((int)px, 0), n - 1), iy = min(max((int)py, 0), n - 1);
            const float* se = td.s_ero + (size_t)iy * n + ix;
            tap[0][l] = __ldg(se);
            tap[1][l] = ix + 1 < n ? __ldg(se + 1) : 0.0f;
            tap[2][l] = iy + 1 < n ? __ldg(se + n) : 0.0f;
            tap[3][l] = (ix + 1 < n && iy + 1 < n) ? __ldg(se + n + 1) : 0.0f;
        }
        sed[h] = bilinear_mix2(bx, by, make_float2(tap[0][0], tap[0][1]), make_float2(tap[1][0], tap[1][1]),
                               make_float2(tap[2][0], tap[2][1]), make_float2(tap[3][0], tap[3][1]));
    }
    st4(td.out[S_SED] + gi0, make_float4(sed[0].x, sed[0].y, sed[1].x, sed[1].y));
}

// One block: the run of tiles k0 .. k1 - 1 (rows of tiles) of strip sx of a
// terrain; `blk` is the block's index within the terrain.
template <int TH>
__device__ __forceinline__ void transport_run(const TerrainHot& td, const CUtensorMap* maps, int blk, int* err) {
    using T = TGeo<TH>;
    extern __shared__ __align__(128) float tr_sm[];
    float* be[2] = {tr_sm, tr_sm + Geo<TH>::T_BOX};
    float* outf = tr_sm + 2 * Geo<TH>::T_BOX;
    __shared__ __align__(8) uint64_t bar[2];
    const StepConsts& c = td.c;
    const int n = c.n;
    const int tiles_y = n / TH;
    const int sx = blk % td.tiles_x, seg = blk / td.tiles_x;
    const int k0 = seg * T::SEG, k1 = min(k0 + T::SEG, tiles_y);
    const int tx0 = sx * TW;
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
    }
    __syncthreads();
    if (tid >= T::TT) {  // ---- gather warps ----
        const int gt = tid - T::TT;
        for (int k = k0; k < k1; ++k)
            for (int q = gt; q < TH * GPR; q += T::GT) gather_group(td, tx0 + 4 * (q % GPR), k * TH + q / GPR);
        // k_hydro of this step has finished (stream order) and the next
        // step's k_hydro starts after this launch: advance the step counter
        if (blk == 0 && gt == 0) *td.step += 1ull;
        return;
    }
    if (!c.thermal) return;
    // ---- talus warps ----
    const int tt = tid;
    auto issue = [&](int k, int stage) {  // thread 0: the eroded rock box of tile row k
        // the buffer's previous contents were read by every talus thread
        // (ordered by the barrier before this call); order those reads
        // before the async-proxy write
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive_expect_tx(&bar[stage], Geo<TH>::T_BOX * sizeof(float));
        tma_load_2d(be[stage], &maps[M_BERO], tx0 - HX, k * TH - 2, &bar[stage]);
    };
    if (tt == 0) issue(k0, 0);
    uint32_t parity = 0;  // bit s: parity of stage s's next completion
    for (int k = k0; k < k1; ++k) {
        const int stage = (k - k0) & 1;
        const bool ok = talus_sync_and<TH>(mbar_wait(&bar[stage], (parity >> stage) & 1u));
        if (!ok) {  // the tile never arrived: record, give the copy one more bounded wait, stop
            if (tt == 0) atomicExch(err, 1);
            mbar_wait(&bar[stage], (parity >> stage) & 1u);
            return;
        }
        parity ^= 1u << stage;
        if (tt == 0 && k + 1 < k1) issue(k + 1, stage ^ 1);
        const int ty0 = k * TH;
        const bool inner = tx0 - HX >= 0 && tx0 + TW + HX <= n && ty0 - 2 >= 0 && ty0 + TH + 2 <= n;
        const int r0 = k == k0 ? 0 : 2;
        if (inner) talus_rows<TH, false>(c, be[stage], outf, tx0, ty0, r0, tt);
        else talus_rows<TH, true>(c, be[stage], outf, tx0, ty0, r0, tt);
        talus_sync<TH>();
        talus_apply<TH>(td, be[stage], outf, tx0, ty0, tt);
        if (k + 1 < k1) {
            talus_sync<TH>();  // every apply has read the outflows
            // rows ty0 + TH - 1 and ty0 + TH become the next tile's rows 0, 1
            for (int i = tt; i < T::PLANES * 2 * RW; i += T::TT) {
                const int pl = i / (2 * RW), r = i % (2 * RW);
                outf[pl * T::OPL + r] = outf[pl * T::OPL + (T::OR - 2) * RW + r];
            }
        }
    }
}

template <int TH>
__global__ void __launch_bounds__(TGeo<TH>::NT, TH == 16 ? 2 : 4) k_transport(const __grid_constant__ BatchParams bp,
                                                                       const CUtensorMap* __restrict__ maps,
                                                                       int* err) {
    const int t = find_terrain(bp.blk0, bp.nterr, blockIdx.x);
    transport_run<TH>(bp.t[t], maps + MAPS_PER_TERRAIN * t, blockIdx.x - bp.blk0[t], err);
}

template <int TH>
__global__ void __launch_bounds__(TGeo<TH>::NT, TH == 16 ? 2 : 4) k_transport1(const __grid_constant__ TerrainDesc td,
                                                                        int* err) {
    transport_run<TH>(td.h, td.maps, blockIdx.x, err);
}

// ---------------------------------------------------------------------------
// tensor maps
// ---------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

bool encode_box(CUtensorMap* map, const float* base, int n, int box_h) {
    std::call_once(g_encode_once, [] {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    if (!g_encode) return false;
    cuuint64_t dims[2] = {(cuuint64_t)n, (cuuint64_t)n};
    cuuint64_t strides[1] = {(cuuint64_t)n * sizeof(float)};
    cuuint32_t box[2] = {(cuuint32_t)RW, (cuuint32_t)box_h};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box,
                          estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace

bool TmaCache::get(const float* base, int n, int box_h, CUtensorMap* out) {
    for (auto& e : entries)
        if (e.base == base && e.n == n && e.box_h == box_h) {
            *out = e.map;
            return true;
        }
    Entry e{base, n, box_h, {}};
    if (!encode_box(&e.map, base, n, box_h)) return false;
    entries.push_back(e);
    *out = e.map;
    return true;
}

bool fused_tile_ok(int n, int th) { return (th == 16 || th == 8) && n % TW == 0 && n % th == 0; }

int fused_tiles(int n, int th) { return (n / TW) * (n / th); }

bool fill_desc(TerrainDesc& d, const TerrainSrc& s, int th, int tile0, TmaCache& cache) {
    TerrainHot& h = d.h;
    h.c = s.c;
    h.rain = s.rain;
    for (int f = 0; f < S_COUNT; ++f) h.out[f] = s.out[f];
    h.u = s.u;
    h.v = s.v;
    h.s_ero = s.s_ero;
    h.b_ero = s.b_ero;
    h.step = s.step;
    h.tiles_x = s.c.n / TW;
    h.tile0 = tile0;
    const int in_fields[H_N] = {S_ROCK, S_WATER, S_SED, S_FL, S_FR, S_FT, S_FB};
    for (int f = 0; f < H_N; ++f)
        if (!cache.get(s.in[in_fields[f]], s.c.n, th + 2, &d.maps[f])) return false;
    return cache.get(s.b_ero, s.c.n, th + 4, &d.maps[M_BERO]);
}

int sweep_blocks(int n, int th) {
    const int seg = th == 16 ? TGeo<16>::SEG : TGeo<8>::SEG;
    return (n / TW) * ((n / th + seg - 1) / seg);
}

namespace {
template <int TH, class K>
void set_transport_smem(K kernel) {
    static std::once_flag once;
    std::call_once(once, [&] {
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TGeo<TH>::SMEM);
    });
}

template <int TH>
void launch_table(const BatchParams& bp, const CUtensorMap* maps, int total_tiles, int* err, cudaStream_t st) {
    int blocks = 0;
    for (int i = 0; i < bp.nterr; ++i) blocks += sweep_blocks(bp.t[i].c.n, TH);
    set_transport_smem<TH>(k_transport<TH>);
    k_hydro<TH><<<total_tiles, Geo<TH>::NTH, 0, st>>>(bp, maps, err);
    k_transport<TH><<<blocks, TGeo<TH>::NT, TGeo<TH>::SMEM, st>>>(bp, maps, err);
    count_launch(2);
}

template <int TH>
void launch_one(const TerrainDesc& td, int* err, cudaStream_t st) {
    set_transport_smem<TH>(k_transport1<TH>);
    k_hydro1<TH><<<fused_tiles(td.h.c.n, TH), Geo<TH>::NTH, 0, st>>>(td, err);
    k_transport1<TH><<<sweep_blocks(td.h.c.n, TH), TGeo<TH>::NT, TGeo<TH>::SMEM, st>>>(td, err);
    count_launch(2);
}
}  // namespace

void launch_fused_table(const BatchParams& bp, const CUtensorMap* maps, int total_tiles, int th, int* err,
                        cudaStream_t st) {
    if (th == 16) launch_table<16>(bp, maps, total_tiles, err, st);
    else launch_table<8>(bp, maps, total_tiles, err, st);
}

void launch_fused_one(const TerrainDesc& td, int th, int* err, cudaStream_t st) {
    if (th == 16) launch_one<16>(td, err, st);
    else launch_one<8>(td, err, st);
}

}  // namespace hg
