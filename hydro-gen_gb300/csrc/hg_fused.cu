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
// Edge tiles (whose box leaves the grid) run either their own copy of the
// tile code or the inner tiles' code with block-uniform edge branches: the
// latter for batches and worlds below 4096² (see hydro_block).
//
// Both kernels are table driven: one launch covers every tile of any number
// of worlds ("terrains") of different sizes and settings.  A block finds its
// terrain by binary search over the terrains' first tiles and reads the terrain's record (step constants, rain
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
//   k_transport stages the eroded rock with a 2-row halo by one TMA load;
//   each thread owns a row group of four horizontally adjacent cells: it
//   computes their eight talus outflows once into shared memory (the ring of
//   interior plus 1 too), applies outflow and inflow, and gathers the four
//   sediment taps of every cell from L2/HBM.
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
    static constexpr int NTH = TH * GPR;                 // one row group per thread in k_transport
    static constexpr int H_RH = TH + 2, H_BOX = RW * H_RH;
    static constexpr int H_RC = ((H_BOX + 31) / 32) * 32;  // 128-byte aligned array stride
    static constexpr int T_RH = TH + 4, T_BOX = RW * T_RH;
    static constexpr int O_RH = TH + 2, O_C = RW * O_RH;   // outflows of interior plus 1
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
// Sets the cells of a staged box that lie outside the grid to v.  The box
// (ROWS x RW cells, row 0 at global row gy0, column 0 at global column
// gx0 = tx0 - HX) reaches past the grid only through its HX outer columns
// on either side and its HALO outer rows on either side, so only those
// are visited (a corner cell twice, with the same value).
template <int ROWS, int HALO, int NTH>
__device__ __forceinline__ void fill_outside(float* box, int gx0, int gy0, int n, float v, int tid) {
    constexpr int SIDE = ROWS * 2 * HX;  // the outer columns of every row
    constexpr int CAP = 2 * HALO * RW;   // the outer rows
    for (int i = tid; i < SIDE + CAP; i += NTH) {
        int r, col;
        if (i < SIDE) {
            r = i / (2 * HX);
            const int k = i % (2 * HX);
            col = k < HX ? k : RW - 2 * HX + k;
        } else {
            const int j = i - SIDE, rr = j / RW;
            col = j % RW;
            r = rr < HALO ? rr : ROWS - 2 * HALO + rr;
        }
        const int gx = gx0 + col, gy = gy0 + r;
        if (gx < 0 || gx >= n || gy < 0 || gy >= n) box[r * RW + col] = v;
    }
}

// EM: 0 inner tile, 1 edge tile (each its own code), 2 either, told at run
// time by edge_rt (one code path for both)
template <int TH, int EM>
__device__ __forceinline__ void hydro_tile(const TerrainHot& td, const CUtensorMap* maps, float* sm, uint64_t* bar,
                                           int tx0, int ty0, bool edge_rt, int* err) {
    const bool EDGE = EM == 2 ? edge_rt : EM == 1;
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
    if (EDGE) {  // water outside the grid (zero-filled by the copy) becomes the shader's
                 // out-of-range height: with rock 0 there, the neighbour's total height
                 // rock + water is exactly FAR_HEIGHT; rock 0 and flux 0 outside are
                 // what the shader reads there too, so neighbour reads need no test
        fill_outside<H_RH, 1, NTH>(sm + H_D * H_RC, gx0, gy0, n, FAR_HEIGHT, tid);
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
        // neighbours outside the grid read rock 0, flux 0 and total height
        // FAR_HEIGHT from the tile (see the fill above); the closed-boundary
        // outflow zeroing runs in edge tiles
        float b = B[si], d1 = D[si];
        float bl = B[si - 1], br = B[si + 1], bb = B[si - RW], bt = B[si + RW];
        float w_c = b + d1;
        float wl = bl + D[si - 1];
        float wr = br + D[si + 1];
        float wt = bt + D[si + RW];
        float wb = bb + D[si - RW];
        FluxOut o = cell_flux(c, x, y, w_c, d1, FL[si], FR[si], FT[si], FB[si], wl, wr, wt, wb, FR[si - 1], FL[si + 1],
                              FB[si + RW], FT[si - RW], EDGE);
        float s = S[si];
        float Kls0 = c.ks_field ? c.dt * __ldg(c.ks_field + gi) : c.Kls0;
        cell_erosion(c, Kls0, o.u, o.v, o.vz, b, s, br, bl, bb, bt);
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

template <int TH, bool SPLIT>
__device__ __forceinline__ void hydro_block(const TerrainHot& td, const CUtensorMap* maps, int tile, int* err) {
    using G = Geo<TH>;
    __shared__ __align__(128) float sm[H_N * G::H_RC];
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    const int n = td.c.n;
    const int tx0 = (tile % td.tiles_x) * TW, ty0 = (tile / td.tiles_x) * TH;
    bool inner = tx0 - HX >= 0 && tx0 + TW + HX <= n && ty0 - 1 >= 0 && ty0 + TH + 1 <= n;
    // Small terrains are mostly edge tiles, interleaved with inner ones on
    // every SM: !SPLIT runs one code path for both (two unrolled copies
    // missed in the instruction cache: 4.6 stalls per issue on an empty
    // instruction buffer, 11 % more time at 256²).  A large world is almost
    // all inner tiles and keeps a copy specialised for them (SPLIT).
    if (!SPLIT) hydro_tile<TH, 2>(td, maps, sm, &bar, tx0, ty0, !inner, err);
    else if (inner) hydro_tile<TH, 0>(td, maps, sm, &bar, tx0, ty0, false, err);
    else hydro_tile<TH, 1>(td, maps, sm, &bar, tx0, ty0, true, err);
}

// Batch form: the terrain records are a kernel parameter (constant bank),
// the block finds its terrain by binary search.
template <int TH>
__global__ void __launch_bounds__(Geo<TH>::NTH) k_hydro(const __grid_constant__ BatchParams bp,
                                                        const CUtensorMap* __restrict__ maps, int* err) {
    const int t = find_terrain(bp.tile0, bp.nterr, blockIdx.x);
    hydro_block<TH, false>(bp.t[t], maps + MAPS_PER_TERRAIN * t, blockIdx.x - bp.tile0[t], err);
}

// Single-world form: the whole descriptor, tensor maps included, is a kernel
// parameter.  SPLIT as for hydro_block: the host picks it by world size.
template <int TH, bool SPLIT>
__global__ void __launch_bounds__(Geo<TH>::NTH) k_hydro1(const __grid_constant__ TerrainDesc td, int* err) {
    hydro_block<TH, SPLIT>(td.h, td.maps, blockIdx.x + td.tile_off, err);
}

// ---------------------------------------------------------------------------
// k_transport: sediment_transport, then thermal_erosion/thermal_transport
// (layer 0).  The eroded rock of the 64 x TH tile and a two-row halo is
// staged by one TMA load.  Each thread owns a row group of four cells,
// evaluated as two f32x2 pairs: it issues the group's sediment taps before
// the tile's TMA wait and mixes them after it, computes talus outflows (the
// ring of interior plus one as pairs of ring cells, then its own group) into
// shared memory, and after the block barrier applies its own outflows and
// its neighbours' inflows.
// ---------------------------------------------------------------------------

// Neighbour rock of the cell at region (rx, ry), global (gx, gy), in
// direction order L, R, T, B, LT, RT, LB, RB (FAR_HEIGHT outside the grid).
template <bool EDGE>
__device__ __forceinline__ void talus_nb(const float* be, int rx, int ry, int gx, int gy, int n, float nb[8]) {
    const int si = ry * RW + rx;
#pragma unroll
    for (int d = 0; d < 8; ++d) {
        bool out = false;
        if (EDGE) {
            const int xx = gx + f_ox[d], yy = gy + f_oy[d];
            out = xx < 0 || xx >= n || yy < 0 || yy >= n;
        }
        nb[d] = out ? FAR_HEIGHT : be[si + f_oy[d] * RW + f_ox[d]];
    }
}

// Talus outflows of two ring cells at once (lanes .x, .y) from the staged
// eroded rock (row 0 = global row gy0, column 0 = global column gx0; at the
// grid's edge the box holds FAR_HEIGHT outside the grid, so a neighbour
// outside reads the shader's out-of-range height); a cell outside the grid
// has none.
__device__ __forceinline__ void pair_outflows(const StepConsts& c, const float* be, int rxa, int rya, int rxb,
                                              int ryb, int gx0, int gy0, bool EDGE, float2 o[8]) {
    const int n = c.n;
    const int gxa = gx0 + rxa, gya = gy0 + rya, gxb = gx0 + rxb, gyb = gy0 + ryb;
    const bool ina = !EDGE || (gxa >= 0 && gxa < n && gya >= 0 && gya < n);
    const bool inb = !EDGE || (gxb >= 0 && gxb < n && gyb >= 0 && gyb < n);
    float na[8], nbb[8];  // the staged box holds FAR_HEIGHT outside the grid
    talus_nb<false>(be, rxa, rya, gxa, gya, n, na);
    talus_nb<false>(be, rxb, ryb, gxb, gyb, n, nbb);
    float2 nb2[8];
#pragma unroll
    for (int d = 0; d < 8; ++d) nb2[d] = make_float2(na[d], nbb[d]);
    cell_thermal_outflows2(c, make_float2(be[rya * RW + rxa], be[ryb * RW + rxb]), nb2, o);
    if (EDGE) {
#pragma unroll
        for (int d = 0; d < 8; ++d) {
            if (!ina) o[d].x = 0.0f;
            if (!inb) o[d].y = 0.0f;
        }
    }
}

// Talus outflows of the row group of four cells at region (rx0, ry) (a row
// of the tile, so inside the grid), as two pairs (cells 0, 1 and 2, 3),
// stored to outf (direction stride o_c, the group's first cell at oi);
// osum[h] receives pair h's 0 - own[0] - ... - own[7].
__device__ __forceinline__ void group_outflows(const StepConsts& c, const float* be, int rx0, int ry, float* outf,
                                               int o_c, int oi, float2 osum[2]) {
    // the group's row is in the grid; outside it the box holds FAR_HEIGHT,
    // so every neighbour is read from the box
    osum[0] = osum[1] = pf(0.0f);
    const int si = ry * RW + rx0;
    const float4 m4 = ld4(be + si - RW), c4 = ld4(be + si), p4 = ld4(be + si + RW);
    const float ml = be[si - RW - 1], mr = be[si - RW + 4];
    const float cl = be[si - 1], cr = be[si + 4];
    const float pl = be[si + RW - 1], pr = be[si + RW + 4];
    float nb[4][8];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        nb[j][0] = j == 0 ? cl : at4(c4, j - 1);
        nb[j][1] = j == 3 ? cr : at4(c4, j + 1);
        nb[j][2] = at4(p4, j);
        nb[j][3] = at4(m4, j);
        nb[j][4] = j == 0 ? pl : at4(p4, j - 1);
        nb[j][5] = j == 3 ? pr : at4(p4, j + 1);
        nb[j][6] = j == 0 ? ml : at4(m4, j - 1);
        nb[j][7] = j == 3 ? mr : at4(m4, j + 1);
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        float2 nb2[8], o[8];
#pragma unroll
        for (int d = 0; d < 8; ++d) nb2[d] = make_float2(nb[2 * h][d], nb[2 * h + 1][d]);
        cell_thermal_outflows2(c, make_float2(at4(c4, 2 * h), at4(c4, 2 * h + 1)), nb2, o);
#pragma unroll
        for (int d = 0; d < 8; ++d) {
            osum[h] = sub2(osum[h], o[d]);
            *reinterpret_cast<float2*>(outf + d * o_c + oi + 2 * h) = o[d];
        }
    }
}

template <int TH, int EM>  // EM as for hydro_tile
__device__ __forceinline__ void transport_tile(const TerrainHot& td, const CUtensorMap* maps, float* be, float* outf,
                                               uint64_t* bar, int tx0, int ty0, bool edge_rt, int* err) {
    const bool EDGE = EM == 2 ? edge_rt : EM == 1;
    using G = Geo<TH>;
    constexpr int O_C = G::O_C;
    const StepConsts& c = td.c;
    const int n = c.n;
    const int tid = threadIdx.x;
    const int gx0 = tx0 - HX, gy0 = ty0 - 2;
    if (c.thermal && tid == 0) {
        mbar_arrive_expect_tx(bar, G::T_BOX * sizeof(float));
        tma_load_2d(be, &maps[M_BERO], gx0, gy0, bar);
    }
    const int iy = tid / GPR, g = tid % GPR;
    const int x0 = tx0 + 4 * g, y = ty0 + iy;
    const size_t gi0 = (size_t)y * n + x0;
    const float4 u4 = __ldg(reinterpret_cast<const float4*>(td.u + gi0));
    const float4 v4 = __ldg(reinterpret_cast<const float4*>(td.v + gi0));

    // sediment_transport: semi-Lagrangian gather of eroded sediment (any
    // reach), two cells per pair.  The taps' loads stay in flight across the
    // tile's TMA wait.
    float2 bx[2], by[2], t00[2], t10[2], t01[2], t11[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        backtrace2(c, x0 + 2 * h, y, make_float2(at4(u4, 2 * h), at4(u4, 2 * h + 1)),
                   make_float2(at4(v4, 2 * h), at4(v4, 2 * h + 1)), bx[h], by[h]);
        float tap[4][2];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            const float px = l ? bx[h].y : bx[h].x, py = l ? by[h].y : by[h].x;
            const int ix = min(max((int)px, 0), n - 1), iy2 = min(max((int)py, 0), n - 1);
            const float* se = td.s_ero + (size_t)iy2 * n + ix;
            tap[0][l] = __ldg(se);
            tap[1][l] = ix + 1 < n ? __ldg(se + 1) : 0.0f;
            tap[2][l] = iy2 + 1 < n ? __ldg(se + n) : 0.0f;
            tap[3][l] = (ix + 1 < n && iy2 + 1 < n) ? __ldg(se + n + 1) : 0.0f;
        }
        t00[h] = make_float2(tap[0][0], tap[0][1]);
        t10[h] = make_float2(tap[1][0], tap[1][1]);
        t01[h] = make_float2(tap[2][0], tap[2][1]);
        t11[h] = make_float2(tap[3][0], tap[3][1]);
    }
    auto finish_sed = [&]() {
        const float2 s0 = bilinear_mix2(bx[0], by[0], t00[0], t10[0], t01[0], t11[0]);
        const float2 s1 = bilinear_mix2(bx[1], by[1], t00[1], t10[1], t01[1], t11[1]);
        st4(td.out[S_SED] + gi0, make_float4(s0.x, s0.y, s1.x, s1.y));
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
    if (EDGE) {  // the box's cells outside the grid (zero-filled by the copy) become the
                 // shader's out-of-range height, so every neighbour read needs no test
        fill_outside<G::T_RH, 2, G::NTH>(be, gx0, gy0, n, FAR_HEIGHT, tid);
        __syncthreads();
    }
    // the taps' loads were issued with the tile's copy: mix them now, before
    // the outflows need the registers
    finish_sed();
    // ---- outflows of the ring of interior plus 1, two cells per thread -----
    // pairs: 32 on the top ring row, 32 on the bottom one, then the left and
    // right ring columns row by row
    {
        constexpr int RINGP = TW + TH + 2;
        for (int q = tid; q < RINGP; q += G::NTH) {
            int rxa, rya, rxb, ryb;
            if (q < TW / 2) { rxa = HX + 2 * q; rya = 1; rxb = rxa + 1; ryb = 1; }
            else if (q < TW) { rxa = HX + 2 * (q - TW / 2); rya = TH + 2; rxb = rxa + 1; ryb = TH + 2; }
            else { rxa = HX - 1; rya = 1 + q - TW; rxb = HX + TW; ryb = rya; }
            float2 o2[8];
            pair_outflows(c, be, rxa, rya, rxb, ryb, gx0, gy0, EDGE, o2);
            const int roa = (rya - 1) * RW + rxa, rob = (ryb - 1) * RW + rxb;
            if (q < TW) {  // horizontally adjacent: one 8-byte store per direction
#pragma unroll
                for (int d = 0; d < 8; ++d) *reinterpret_cast<float2*>(outf + d * O_C + roa) = o2[d];
            } else {
#pragma unroll
                for (int d = 0; d < 8; ++d) {
                    outf[d * O_C + roa] = o2[d].x;
                    outf[d * O_C + rob] = o2[d].y;
                }
            }
        }
    }
    // ---- outflows of the interior row groups (one per thread) --------------
    // The thread's own outflow sums (cell_thermal_apply's sum = 0 - own[0] -
    // ... - own[7]) stay in registers.
    const int rx0 = HX + 4 * g, ry = 2 + iy;  // region coords of the group's first cell
    const int oi = (ry - 1) * RW + rx0;
    float2 osum[2];
    group_outflows(c, be, rx0, ry, outf, O_C, oi, osum);
    __syncthreads();
    // ---- thermal_transport: own outflows out, neighbours' outflows in -------
    // (cell_thermal_apply's operations: in_flux = in[0] + ... + in[7] from 0,
    // sum = 0 - own[0] - ... - own[7], rock = b + (sum + in_flux))
    {
        // inflow from direction d = neighbour (dx, dy)'s outflow toward this
        // cell.  Rows of outflows are read as aligned float4 (the group's own
        // four columns); the column left (right) of the group comes from the
        // neighbouring group in the warp, lane - 1 (+ 1), or at the tile edge
        // from the ring column.
        const unsigned FULL = 0xffffffffu;
        const bool first = g == 0, last = g == GPR - 1;
        // left neighbour's direction-dl outflow and right neighbour's
        // direction-dr outflow in the row at offset `off`, as cell pairs
        auto row_in = [&](int dl, int dr, int off, float2 in[2][2]) {
            const float4 a = ld4(outf + dl * O_C + oi + off), b = ld4(outf + dr * O_C + oi + off);
            float pa = __shfl_up_sync(FULL, a.w, 1);
            float nb = __shfl_down_sync(FULL, b.x, 1);
            if (first) pa = outf[dl * O_C + oi + off - 1];
            if (last) nb = outf[dr * O_C + oi + off + 4];
            in[0][0] = make_float2(pa, a.x);
            in[0][1] = make_float2(a.y, a.z);
            in[1][0] = make_float2(b.y, b.z);
            in[1][1] = make_float2(b.w, nb);
        };
        float2 inf[2] = {pf(0.0f), pf(0.0f)};
        auto acc = [&](const float2 v[2]) {
            inf[0] = add2(inf[0], v[0]);
            inf[1] = add2(inf[1], v[1]);
        };
        {
            float2 in[2][2];
            row_in(1, 0, 0, in);  // L neighbour's R, R neighbour's L
            acc(in[0]);
            acc(in[1]);
        }
        {
            const float4 inT = ld4(outf + 3 * O_C + oi + RW);  // top neighbour's B
            const float4 inB = ld4(outf + 2 * O_C + oi - RW);  // bottom neighbour's T
            const float2 t[2] = {make_float2(inT.x, inT.y), make_float2(inT.z, inT.w)};
            const float2 bb[2] = {make_float2(inB.x, inB.y), make_float2(inB.z, inB.w)};
            acc(t);
            acc(bb);
        }
        {
            float2 in[2][2];
            row_in(7, 6, RW, in);  // row above: LT neighbour's RB, RT neighbour's LB
            acc(in[0]);
            acc(in[1]);
        }
        {
            float2 in[2][2];
            row_in(5, 4, -RW, in);  // row below: LB neighbour's RT, RB neighbour's LT
            acc(in[0]);
            acc(in[1]);
        }
        const float4 b4 = ld4(be + ry * RW + rx0);
        const float2 r0 = add2(make_float2(b4.x, b4.y), add2(osum[0], inf[0]));
        const float2 r1 = add2(make_float2(b4.z, b4.w), add2(osum[1], inf[1]));
        st4(td.out[S_ROCK] + gi0, make_float4(r0.x, r0.y, r1.x, r1.y));
    }
}

template <int TH, bool SPLIT>
__device__ __forceinline__ void transport_block(const TerrainHot& td, const CUtensorMap* maps, int tile, int first_tile,
                                                int* err) {
    using G = Geo<TH>;
    __shared__ __align__(128) float be[G::T_BOX];
    __shared__ __align__(16) float outf[8 * G::O_C];
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    const int n = td.c.n;
    const int tx0 = (tile % td.tiles_x) * TW, ty0 = (tile / td.tiles_x) * TH;
    bool inner = tx0 - HX >= 0 && tx0 + TW + HX <= n && ty0 - 2 >= 0 && ty0 + TH + 2 <= n;
    // one code path for a batch, an inner copy for a single world (see hydro_block)
    if (!SPLIT) transport_tile<TH, 2>(td, maps, be, outf, &bar, tx0, ty0, !inner, err);
    else if (inner) transport_tile<TH, 0>(td, maps, be, outf, &bar, tx0, ty0, false, err);
    else transport_tile<TH, 1>(td, maps, be, outf, &bar, tx0, ty0, true, err);
    // k_hydro of this step has finished (stream order) and the next step's
    // k_hydro starts after this launch: advance the terrain's step counter
    if (tile == first_tile && threadIdx.x == 0) *td.step += 1ull;
}

template <int TH>
__global__ void __launch_bounds__(Geo<TH>::NTH, TH == 16 ? 4 : 6) k_transport(const __grid_constant__ BatchParams bp,
                                                            const CUtensorMap* __restrict__ maps, int* err) {
    const int t = find_terrain(bp.tile0, bp.nterr, blockIdx.x);
    transport_block<TH, false>(bp.t[t], maps + MAPS_PER_TERRAIN * t, blockIdx.x - bp.tile0[t], 0, err);
}

template <int TH, bool SPLIT>
__global__ void __launch_bounds__(Geo<TH>::NTH, TH == 16 ? 4 : 6) k_transport1(const __grid_constant__ TerrainDesc td, int* err) {
    transport_block<TH, SPLIT>(td.h, td.maps, blockIdx.x + td.tile_off, td.tile_off, err);
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
    d.tile_off = 0;
    const int in_fields[H_N] = {S_ROCK, S_WATER, S_SED, S_FL, S_FR, S_FT, S_FB};
    for (int f = 0; f < H_N; ++f)
        if (!cache.get(s.in[in_fields[f]], s.c.n, th + 2, &d.maps[f])) return false;
    return cache.get(s.b_ero, s.c.n, th + 4, &d.maps[M_BERO]);
}

void launch_fused_table(const BatchParams& bp, const CUtensorMap* maps, int total_tiles, int th, int* err,
                        cudaStream_t st) {
    if (th == 16) {
        k_hydro<16><<<total_tiles, Geo<16>::NTH, 0, st>>>(bp, maps, err);
        k_transport<16><<<total_tiles, Geo<16>::NTH, 0, st>>>(bp, maps, err);
    } else {
        k_hydro<8><<<total_tiles, Geo<8>::NTH, 0, st>>>(bp, maps, err);
        k_transport<8><<<total_tiles, Geo<8>::NTH, 0, st>>>(bp, maps, err);
    }
    count_launch(2);
}

// Worlds from this side up keep separate inner and edge code (edge tiles are
// under 4 % of a 4096² launch at tile height 16); smaller ones, where edge
// tiles are 8 % (2048²) to 56 % (256²) of the launch, run one code path.
constexpr int SPLIT_MIN_N = 4096;

template <int TH, bool SPLIT>
void launch_one(const TerrainDesc& td, int tiles, int* err, cudaStream_t st) {
    k_hydro1<TH, SPLIT><<<tiles, Geo<TH>::NTH, 0, st>>>(td, err);
    k_transport1<TH, SPLIT><<<tiles, Geo<TH>::NTH, 0, st>>>(td, err);
}

// One kernel of the fused step (which 0: k_hydro, 1: k_transport) over the
// `tiles` tiles from tile_lo on (whole tile rows: a row slab's).
template <int TH, bool SPLIT>
void launch_half(const TerrainDesc& td, int which, int tiles, int* err, cudaStream_t st) {
    if (which == 0) k_hydro1<TH, SPLIT><<<tiles, Geo<TH>::NTH, 0, st>>>(td, err);
    else k_transport1<TH, SPLIT><<<tiles, Geo<TH>::NTH, 0, st>>>(td, err);
}

void launch_fused_half(const TerrainDesc& td0, int th, int which, int tile_lo, int tiles, int* err,
                       cudaStream_t st) {
    if (tiles <= 0) return;
    TerrainDesc td = td0;
    td.tile_off = tile_lo;
    const bool split = td.h.c.n >= SPLIT_MIN_N;
    if (th == 16) {
        if (split) launch_half<16, true>(td, which, tiles, err, st);
        else launch_half<16, false>(td, which, tiles, err, st);
    } else {
        if (split) launch_half<8, true>(td, which, tiles, err, st);
        else launch_half<8, false>(td, which, tiles, err, st);
    }
    count_launch();
}

void launch_fused_one(const TerrainDesc& td, int th, int* err, cudaStream_t st) {
    const int tiles = fused_tiles(td.h.c.n, th);
    const bool split = td.h.c.n >= SPLIT_MIN_N;
    if (th == 16) {
        if (split) launch_one<16, true>(td, tiles, err, st);
        else launch_one<16, false>(td, tiles, err, st);
    } else {
        if (split) launch_one<8, true>(td, tiles, err, st);
        else launch_one<8, false>(td, tiles, err, st);
    }
    count_launch(2);
}

}  // namespace hg
