// Reverse-mode adjoint of the one-layer grid step (talus passes included).
//
// One reversed step j works on the step's input state X_j, the step's
// forward intermediates kept by the segment recompute (velocity u, v and the
// eroded sediment se of every cell: the fused forward step writes them
// anyway) and the adjoint A of the step's outputs.  The adjoint of a state is
// kept as each cell's own terms plus ten packet fields that carry the terms
// of its neighbours' inputs; a reader adds the neighbours' packets in a
// fixed order (deterministic), so no separate gather pass runs.  One kernel
// per step:
//   k_adj_cell      TMA-staged 64 x 4 tiles of X_j with a one-cell halo,
//                   this step's rain added in shared memory; one thread per
//                   cell gathers the cell's adjoint inputs while the tile
//                   flies, recomputes the forward flux and erosion (the
//                   operations of hg_device.cuh, so every branch is the
//                   forward's) and reverses them; it writes its own terms
//                   and packets, accumulates the Ks gradient and clears its
//                   sediment-adjoint cell (double buffer); then, with the
//                   cell's sediment adjoint of step j - 1 now final, it
//                   reverses that step's semi-Lagrangian gather: a scatter
//                   to the back-trace's four taps (atomicAdd: the taps are
//                   data dependent) and the back-trace velocity adjoint
//   k_adj_sediment  the same scatter on its own, for a segment's last step
//                   (its intermediates exist only after the recompute)
//   k_adj_final     the gathered rock adjoint of the first state
//   k_adj_thermal   the talus passes reversed: gathers the output rock's
//                   adjoint over its box from own terms and packets while
//                   the eroded rock's box flies, and yields the adjoint of
//                   the eroded rock, which k_adj_cell then takes
//
// Subgradients: max(0, x) and min(1, q) pass the derivative of the taken
// argument (ties take the constant side), clamps pass 0 when clamped,
// dissolve/deposit/exhaustion use the taken branch, floor() is locally
// constant, and in water films below FILM_DEPTH the velocity and the flux
// scale are locally constant.  The formulas follow the shaders cited in hg_device.cuh.  The
// reversed arithmetic divides through correctly rounded reciprocals
// (x * (1/y), within two ulps of x / y); the recomputed forward keeps IEEE
// division, so its values and branches are the forward's own.
#include "hg_internal.h"
#include "hg_tma.cuh"

namespace hg {

namespace {

constexpr int BX = 32, BY = 8;
__device__ __forceinline__ size_t at(int n, int x, int y) { return (size_t)y * n + x; }

// Water films thinner than this (the depth below which the erosion ignores
// the velocity, glsl/hydro_erosion.glsl:45-52) pass no adjoint through the
// velocity (u = flux difference / depth) or the flux scale (K = depth /
// outflow): both derivatives grow like 1/depth and overflow float in the
// films that intermittent rain leaves (depths reach 1e-35), where they carry
// no usable gradient anyway.
constexpr float FILM_DEPTH = 5e-4f;

// ---- sediment_transport reversed ------------------------------------------------
// Cell (x, y) of a step whose output sediment adjoint is `a`: scatter to the
// back-trace taps of dse, back-trace velocity adjoint into du, dv.
__device__ __forceinline__ void sediment_adjoint(const StepConsts& c, const AdjSlot& sl, int x, int y, size_t i,
                                                 float a, float ui, float vi, float* dse, float* du, float* dv) {
    const int n = c.n;
    const float maxc = (float)(n - 1);
    float rx = (float)x - ui * c.dt, ry = (float)y - vi * c.dt;
    float px = gclamp(rx, 0.0f, maxc), py = gclamp(ry, 0.0f, maxc);
    int ix = min(max((int)px, 0), n - 1), iy = min(max((int)py, 0), n - 1);
    float fx = px - floorf(px), fy = py - floorf(py);
    auto S = [&](int xx, int yy) -> float { return (xx < n && yy < n) ? sl.se[at(n, xx, yy)] : 0.0f; };
    auto add = [&](int xx, int yy, float v) {
        if (xx < n && yy < n && v != 0.0f) atomicAdd(dse + at(n, xx, yy), v);
    };
    add(ix, iy, a * (1.0f - fx) * (1.0f - fy));
    add(ix + 1, iy, a * fx * (1.0f - fy));
    add(ix, iy + 1, a * (1.0f - fx) * fy);
    add(ix + 1, iy + 1, a * fx * fy);
    float s00 = S(ix, iy), s10 = S(ix + 1, iy), s01 = S(ix, iy + 1), s11 = S(ix + 1, iy + 1);
    float dfx = (s10 - s00) * (1.0f - fy) + (s11 - s01) * fy;
    float dfy = (s01 * (1.0f - fx) + s11 * fx) - (s00 * (1.0f - fx) + s10 * fx);
    du[i] = (rx > 0.0f && rx < maxc) ? a * dfx * (-c.dt) : 0.0f;
    dv[i] = (ry > 0.0f && ry < maxc) ? a * dfy * (-c.dt) : 0.0f;
}

__global__ void k_adj_sediment(StepConsts c, AdjSlot sl, const float* __restrict__ as_, float* __restrict__ dse,
                               float* __restrict__ du, float* __restrict__ dv) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= c.n || y >= c.n) return;
    size_t i = at(c.n, x, y);
    sediment_adjoint(c, sl, x, y, i, as_[i], sl.u[i], sl.v[i], dse, du, dv);
}

// Gathered adjoint of a state at cell i: own terms plus the neighbours'
// packets (L, R, T, B neighbours, fixed order).
// ROCK false leaves ab alone (the caller has the rock adjoint from elsewhere)
// and skips the loads only it needs
template <bool ROCK = true>
__device__ __forceinline__ void adj_view_at(const AdjView& A, int n, int x, int y, size_t i, float& ab, float& ad,
                                            float af[4]) {
    // w = rock + water: a neighbour's height difference toward this cell
    // (its direction opposite to ours) enters with a minus sign
    float nbw = 0.0f;
    if (x > 0) nbw += A.pdh[1][i - 1];      // left neighbour's R
    if (x < n - 1) nbw += A.pdh[0][i + 1];  // right neighbour's L
    if (y < n - 1) nbw += A.pdh[3][i + n];  // top neighbour's B
    if (y > 0) nbw += A.pdh[2][i - n];      // bottom neighbour's T
    if (ROCK) {
        float nrm = 0.0f;  // terrain-normal terms of the neighbours
        if (x > 0) nrm += A.pdx[i - 1];
        if (x < n - 1) nrm -= A.pdx[i + 1];
        if (y > 0) nrm += A.pdz[i - n];
        if (y < n - 1) nrm -= A.pdz[i + n];
        ab = (A.b[i] - nbw) + nrm;
    }
    ad = A.d[i] - nbw;
#pragma unroll
    for (int d = 0; d < 4; ++d) af[d] = A.f[d][i];
    if (x > 0) af[0] += A.pin[1][i - 1];      // left neighbour's inflow from me
    if (x < n - 1) af[1] += A.pin[0][i + 1];  // right neighbour's inflow from me
    if (y < n - 1) af[2] += A.pin[3][i + n];  // top neighbour's inflow from me
    if (y > 0) af[3] += A.pin[2][i - n];      // bottom neighbour's inflow from me
}

// The gathered rock adjoint alone, with adj_view_at's operations and order.
__device__ __forceinline__ float adj_rock_at(const AdjView& A, int n, int x, int y, size_t i) {
    float nbw = 0.0f;
    if (x > 0) nbw += A.pdh[1][i - 1];
    if (x < n - 1) nbw += A.pdh[0][i + 1];
    if (y < n - 1) nbw += A.pdh[3][i + n];
    if (y > 0) nbw += A.pdh[2][i - n];
    float nrm = 0.0f;
    if (x > 0) nrm += A.pdx[i - 1];
    if (x < n - 1) nrm -= A.pdx[i + 1];
    if (y > 0) nrm += A.pdz[i - n];
    if (y < n - 1) nrm -= A.pdz[i + n];
    return (A.b[i] - nbw) + nrm;
}

// ---- k_adj_cell ------------------------------------------------------------------
constexpr int TW = 64, TH = 4, HX = 4, RW = TW + 2 * HX, NTH = TW * TH;
constexpr int H_RH = TH + 2, H_BOX = RW * H_RH, H_RC = ((H_BOX + 31) / 32) * 32;
enum { X_B = 0, X_D, X_S, X_FL, X_FR, X_FT, X_FB, X_N };

// Forward flux of one cell with the intermediates its adjoint needs: the
// operations of cell_flux (hg_device.cuh), so every branch is the forward's.
// Directions L, R, T, B; wn[] neighbour totals, in[] neighbours' facing flux.
struct FluxFwd {
    float g[4];
    bool live[4];
    float sum_out, den, K, arg, vz, u, v;
    bool scaled;
};
__device__ __forceinline__ FluxFwd flux_fwd(const StepConsts& c, int x, int y, float w_c, float d1, const float f[4],
                                            const float wn[4], const float in[4], bool border) {
    FluxFwd o;
    float ft[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        ft[k] = c.EK * f[k] + c.dt * (c.G * (w_c - wn[k]));
        o.g[k] = gmax(0.0f, ft[k]);
        o.live[k] = ft[k] > 0.0f;
    }
    if (border) {
        if (x <= 0) { o.g[0] = 0.0f; o.live[0] = false; }
        else if (x >= c.n - 1) { o.g[1] = 0.0f; o.live[1] = false; }
        if (y <= 0) { o.g[3] = 0.0f; o.live[3] = false; }
        else if (y >= c.n - 1) { o.g[2] = 0.0f; o.live[2] = false; }
    }
    float sum_in = in[0] + in[1] + in[2] + in[3];
    o.sum_out = o.g[0] + o.g[1] + o.g[2] + o.g[3];
    o.den = o.sum_out * c.dt;
    o.scaled = false;
    o.K = 1.0f;
    if (!(d1 >= o.den)) {
        float q = d1 / o.den;
        if (q < 1.0f) { o.scaled = true; o.K = q; }
    }
    o.arg = d1 + c.dt * (sum_in - o.sum_out * o.K);
    float d2 = gmax(0.0f, o.arg);
    o.vz = d1 + d2;
    if (o.vz > 0.0f) {
        o.u = (in[0] - f[0] + f[1] - in[1]) / o.vz;
        o.v = (in[3] - f[3] + f[2] - in[2]) / o.vz;
    } else {
        o.u = 0.0f; o.v = 0.0f;
    }
    return o;
}

template <bool EDGE>
__device__ __forceinline__ void adj_tile(const AdjCellArgs& a, float* sm, uint64_t* bar, int tx0, int ty0,
                                         int* err) {
    const StepConsts& c = a.c;
    const RainStep& r = a.rain;
    const int n = c.n;
    const int tid = threadIdx.x;
    const int gx0 = tx0 - HX, gy0 = ty0 - 1;
    if (tid == 0) {
        mbar_arrive_expect_tx(bar, X_N * H_BOX * sizeof(float));
#pragma unroll
        for (int f = 0; f < X_N; ++f) tma_load_2d(sm + f * H_RC, &a.maps[f], gx0, gy0, bar);
    }
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
    // the cell's adjoint inputs, loaded while the tile flies
    const int ix = tid % TW, iy = tid / TW;
    const int x = tx0 + ix, y = ty0 + iy;
    const size_t i = (size_t)y * n + x;
    float ab, ad, af[4];
    if (a.gbe) {  // thermal on: the eroded rock's adjoint (k_adj_thermal)
        ab = a.gbe[i];
        adj_view_at<false>(a.A, n, x, y, i, ab, ad, af);
    } else {
        adj_view_at(a.A, n, x, y, i, ab, ad, af);
    }
    const float as = a.dse[i];
    const float DUs = a.du[i], DVs = a.dv[i];
    const float Ks_i = c.ks_field ? c.ks_field[i] : c.Ks0;
    // step j - 1's velocity for its sediment reversal at the end
    const float pu = a.scatter_prev ? a.prev.u[i] : 0.0f, pv = a.scatter_prev ? a.prev.v[i] : 0.0f;
    bool ok = __syncthreads_and(mbar_wait(bar, 0));
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        mbar_wait(bar, 0);
        return;
    }
    if (r.active) {
        float* D = sm + X_D * H_RC;
#pragma unroll
        for (int k = 0; k < RGK; ++k) {
            int q = tid + k * NTH;
            if (q >= RG) continue;
            int rx = (q % (RW / 4)) * 4, ry = q / (RW / 4);
            int gx = gx0 + rx, gy = gy0 + ry;
            if (EDGE && !(gx >= 0 && gx < n && gy >= 0 && gy < n)) continue;
            float* p = D + ry * RW + rx;
            p[0] += rain_incr(r, words[k][0]);
            p[1] += rain_incr(r, words[k][1]);
            p[2] += rain_incr(r, words[k][2]);
            p[3] += rain_incr(r, words[k][3]);
        }
    }
    __syncthreads();
    const float* B = sm + X_B * H_RC;
    const float* D = sm + X_D * H_RC;
    const float* S = sm + X_S * H_RC;
    const float* F[4] = {sm + X_FL * H_RC, sm + X_FR * H_RC, sm + X_FT * H_RC, sm + X_FB * H_RC};
    {
        const int si = (1 + iy) * RW + HX + ix;
        const bool has_l = !EDGE || x > 0, has_r = !EDGE || x < n - 1;
        const bool has_b = !EDGE || y > 0, has_t = !EDGE || y < n - 1;
        // ---- forward recompute: flux --------------------------------------
        const float b = B[si], d1 = D[si];
        const float bl = B[si - 1], br = B[si + 1], bb = B[si - RW], bt = B[si + RW];
        const float f[4] = {F[0][si], F[1][si], F[2][si], F[3][si]};
        const float wn[4] = {has_l ? bl + D[si - 1] : FAR_HEIGHT, has_r ? br + D[si + 1] : FAR_HEIGHT,
                             has_t ? bt + D[si + RW] : FAR_HEIGHT, has_b ? bb + D[si - RW] : FAR_HEIGHT};
        const float in[4] = {has_l ? F[1][si - 1] : 0.0f, has_r ? F[0][si + 1] : 0.0f,
                             has_t ? F[3][si + RW] : 0.0f, has_b ? F[2][si - RW] : 0.0f};
        const FluxFwd fw = flux_fwd(c, x, y, b + d1, d1, f, wn, in, EDGE);
        // ---- forward recompute: erosion speed and tilt ---------------------
        const float u = fw.u, v = fw.v, vz = fw.vz;
        const float len = sqrtf(u * u + v * v);
        float ero = len, dero_dlen = 1.0f, dero_dvz = 0.0f;
        if (vz < 1e-3f) {
            float dd = gmax(5e-4f, vz);
            float tr = (dd - 1e-3f) / (5e-4f - 1e-3f);
            float t = gclamp(tr, 0.0f, 1.0f);
            float sm3 = t * t * (3.0f - 2.0f * t);
            ero = gmix(len, 0.0f, sm3);
            dero_dlen = 1.0f - sm3;
            // d(smoothstep)/d(vz): 6 t (1 - t) / (5e-4 - 1e-3)
            if (vz > 5e-4f && tr > 0.0f && tr < 1.0f) dero_dvz = len * 6.0f * t * (1.0f - t) * 2000.0f;
        }
        const float ebr = has_r ? br : 0.0f, ebl = has_l ? bl : 0.0f;
        const float ebt = has_t ? bt : 0.0f, ebb = has_b ? bb : 0.0f;
        const float dx = ebr - ebl, dz = ebt - ebb;
        const float cx = dx * 2.0f - 0.0f * dz, cz = 2.0f * dz - dx * 0.0f;
        const float L3 = sqrtf(cx * cx + 16.0f + cz * cz);
        const float ny = -4.0f / L3;
        const float sin_a = fabsf(sqrtf(1.0f - ny * ny));
        const float sa = gmax(0.02f, sin_a);
        const float craw = c.Kc * sa * ero;
        const float cc = gmax(0.0f, craw);
        const float Kls = c.dt * Ks_i, Kld = c.Kld0, s = S[si];
        // ---- erosion reversed ----------------------------------------------
        a.dse[i] = 0.0f;  // free for the step after next
        float gb, gs, gc = 0.0f, gKs = 0.0f;
        if (cc > 0.0f && !(c.Kls1 * cc > 0.0f)) {  // the empty dirt layer ends the layer loop: identity
            gb = ab;
            gs = as;
        } else if (cc > s) {
            float del = Kls * (cc - s);
            if (b - del < 0.0f) {  // rock exhausted: b' = 0, s' = s + b
                gb = as;
                gs = as;
            } else {
                gb = ab;
                gs = ab * Kls + as * (1.0f - Kls);
                gc = (as - ab) * Kls;
                gKs = (as - ab) * (cc - s);
            }
        } else {
            gb = ab;
            gs = ab * Kld + as * (1.0f - Kld);
            gc = (as - ab) * Kld;
        }
        if (gKs != 0.0f) a.dks[i] += gKs * c.dt;
        float pdx = 0.0f, pdz = 0.0f, due = 0.0f, dve = 0.0f, gvz = 0.0f;
        if (craw > 0.0f) {
            float gsa = gc * c.Kc * ero, gero = gc * c.Kc * sa;
            if (sin_a > 0.02f) {
                const float r3 = __frcp_rn(L3);
                float gny = gsa * (-ny * __frcp_rn(sin_a));
                float gL3 = gny * (4.0f * r3 * r3);
                pdx = gL3 * 4.0f * dx * r3;
                pdz = gL3 * 4.0f * dz * r3;
            }
            float glen = gero * dero_dlen;
            gvz = gero * dero_dvz;
            if (len > 0.0f) {
                const float rl = __frcp_rn(len);
                due = glen * u * rl;
                dve = glen * v * rl;
            }
        }
        // ---- flux reversed -------------------------------------------------
        const float DU = DUs + due, DV = DVs + dve;
        float gin[4] = {0.0f, 0.0f, 0.0f, 0.0f}, gfown[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (vz >= FILM_DEPTH) {  // thinner films: velocity locally constant
            const float rv = __frcp_rn(vz);
            float gu = DU * rv, gv = DV * rv;
            gin[0] += gu; gin[1] -= gu;
            gfown[0] -= gu; gfown[1] += gu;
            gin[3] += gv; gin[2] -= gv;
            gfown[3] -= gv; gfown[2] += gv;
            gvz -= (DU * u + DV * v) * rv;
        }
        float gd1 = gvz, gd2 = gvz + ad * c.evap;
        float garg = fw.arg > 0.0f ? gd2 : 0.0f;
        gd1 += garg;
        float gsum_in = c.dt * garg, gsum_outK = -c.dt * garg;
#pragma unroll
        for (int d = 0; d < 4; ++d) gin[d] += gsum_in;
        float gK = gsum_outK * fw.sum_out, gsum_out = gsum_outK * fw.K;
#pragma unroll
        for (int d = 0; d < 4; ++d) gK += af[d] * fw.g[d];
        float gg[4];
#pragma unroll
        for (int d = 0; d < 4; ++d) gg[d] = af[d] * fw.K + gsum_out;
        if (fw.scaled && d1 >= FILM_DEPTH) {  // thinner films: K locally constant
            const float rd = __frcp_rn(fw.den);
            gd1 += gK * rd;
            float gden = -gK * d1 * rd * rd;
#pragma unroll
            for (int d = 0; d < 4; ++d) gg[d] += gden * c.dt;
        }
        float gw = 0.0f;
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            float gdh = 0.0f;
            if (fw.live[d]) {
                gfown[d] += c.EK * gg[d];
                gdh = c.dt * c.G * gg[d];
                gw += gdh;
            }
            a.pdh[d][i] = gdh;
            a.pin[d][i] = gin[d];
            a.rf[d][i] = gfown[d];
        }
        a.pdx[i] = pdx;
        a.pdz[i] = pdz;
        a.rb[i] = gb + gw;
        a.rd[i] = gw + gd1;
        a.rs[i] = gs;
        // ---- sediment_transport of step j - 1 reversed ----------------------
        if (a.scatter_prev) sediment_adjoint(c, a.prev, x, y, i, gs, pu, pv, a.dse_prev, a.du, a.dv);
    }
}

__global__ void __launch_bounds__(NTH) k_adj_cell(const __grid_constant__ AdjCellArgs a, int* err) {
    __shared__ __align__(128) float sm[X_N * H_RC];
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    const int n = a.c.n;
    const int tiles_x = n / TW;
    const int tx0 = (blockIdx.x % tiles_x) * TW, ty0 = (blockIdx.x / tiles_x) * TH;
    bool inner = tx0 - HX >= 0 && tx0 + TW + HX <= n && ty0 - 1 >= 0 && ty0 + TH + 1 <= n;
    if (inner) adj_tile<false>(a, sm, &bar, tx0, ty0, err);
    else adj_tile<true>(a, sm, &bar, tx0, ty0, err);
}

// ---- k_adj_final -----------------------------------------------------------------
__global__ void k_adj_final(int n, AdjView A, float* __restrict__ out_b) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= n || y >= n) return;
    out_b[at(n, x, y)] = adj_rock_at(A, n, x, y, at(n, x, y));
}

// ---- k_adj_thermal ---------------------------------------------------------------
// Reverse of thermal_erosion + thermal_transport (layer 0): from the adjoint
// A of the rock after the talus passes to the adjoint G of the eroded rock.
// rock' = b + sum_k in_k - sum_k o_k, o_k = S dh_k / bk for the marked
// directions, S = dt Kspeed sharp^3 H / 2.  With g_k = A(neighbour k) - A(c):
//   dL/ddh_j = S/bk (g_j - gbar) for marked j, gbar = sum_k g_k dh_k / bk
//   dL/dS = gbar; H = min(b, max dh) and the steepest marked slope pass
//   their derivative to the direction that attains them (the first one in
//   direction order); the marks themselves are locally constant.
// dh_j = b(c) - b(neighbour j): +dL/ddh_j to the cell, - to the neighbour.
// 64 x 16 tiles of 512 threads (the ring's share of the recomputed cells is
// 16 % against 29 % for 64 x 8: 3 % less time); the per-cell terms of the
// tile and its one-cell ring go through shared memory (54 KB, dynamic), from
// a TMA box of the eroded rock and the gathered A, both with a two-cell halo.
constexpr int TT_H = 16, TT_NTH = 512;
constexpr int TT_RW = TW + 2 * HX, TT_BH = TT_H + 4, TT_BOX = TT_RW * TT_BH;
constexpr int TT_BRC = ((TT_BOX + 31) / 32) * 32;
constexpr int TT_CW = TW + 2, TT_CH = TT_H + 2, TT_NC = TT_CW * TT_CH;  // tile + ring
// direction k = L, R, T, B, LT, RT, LB, RB -> offset
__host__ __device__ constexpr int tt_ox(int k) { return (k == 0 || k == 4 || k == 6) ? -1 : (k == 1 || k == 5 || k == 7) ? 1 : 0; }
__host__ __device__ constexpr int tt_oy(int k) { return (k == 2 || k == 4 || k == 5) ? 1 : (k == 3 || k == 6 || k == 7) ? -1 : 0; }

struct ThermalArgs {
    CUtensorMap map_b;  // eroded rock of the step (box TT_RW x TT_BH)
    AdjView A;          // adjoint of the step's output (own terms + packets)
    StepConsts c;
    float* g;           // out: adjoint of the eroded rock
};

template <bool EDGE>
__device__ __forceinline__ void thermal_tile(const ThermalArgs& ta, float* bs, float* as, float* gd, uint64_t* bar,
                                             int tx0, int ty0, int* err) {
    const StepConsts& c = ta.c;
    const int n = c.n, tid = threadIdx.x;
    const int gx0 = tx0 - HX, gy0 = ty0 - 2;
    if (tid == 0) {
        mbar_arrive_expect_tx(bar, TT_BOX * sizeof(float));
        tma_load_2d(bs, &ta.map_b, gx0, gy0, bar);
    }
    // while the eroded rock flies: the gathered adjoint A of the output rock
    // over the region's columns 2 .. TT_RW - 3 (the tile, its ring and their
    // neighbours), 0 outside the grid
#pragma unroll 1
    for (int q = tid; q < (TT_RW - 4) * TT_BH; q += TT_NTH) {
        const int rx = 2 + q % (TT_RW - 4), ry = q / (TT_RW - 4);
        const int x = gx0 + rx, y = gy0 + ry;
        float v = 0.0f;
        if (!EDGE || (x >= 0 && x < n && y >= 0 && y < n)) v = adj_rock_at(ta.A, n, x, y, (size_t)y * n + x);
        as[ry * TT_RW + rx] = v;
    }
    bool ok = __syncthreads_and(mbar_wait(bar, 0));
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        mbar_wait(bar, 0);
        return;
    }
    // per-cell terms of the tile and its ring: gd[k * TT_NC + q] = dL/ddh_k,
    // gd[8 * TT_NC + q] = the cell's own term (dL/db through H, plus sum_k dL/ddh_k)
#pragma unroll 1
    for (int q = tid; q < TT_NC; q += TT_NTH) {
        const int rx = q % TT_CW - 1, ry = q / TT_CW - 1;
        const int x = tx0 + rx, y = ty0 + ry;
        float gdh[8] = {0, 0, 0, 0, 0, 0, 0, 0}, own = 0.0f;
        if (!EDGE || (x >= 0 && x < n && y >= 0 && y < n)) {
            const int si = (ry + 2) * TT_RW + HX + rx;
            const float b = bs[si];
            float dh[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                bool out = EDGE && (x + tt_ox(k) < 0 || x + tt_ox(k) >= n || y + tt_oy(k) < 0 || y + tt_oy(k) >= n);
                dh[k] = b - (out ? FAR_HEIGHT : bs[si + tt_oy(k) * TT_RW + tt_ox(k)]);
            }
            // the forward's values (cell_thermal_outflows' operations)
            float Hmax = 0.0f;
            int jh = -1;
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (dh[k] > Hmax) { Hmax = dh[k]; jh = k; }
            const float H = gmin(b, Hmax);
            float bk = 0.0f, max_cross = 0.0f, max_diag = 0.0f;
            int jc = -1, jd = -1;
            bool mk[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                mk[k] = dh[k] >= (k < 4 ? c.talus_x_cross : c.talus_b_diag);
                if (mk[k]) {
                    bk += dh[k];
                    if (k < 4) { if (dh[k] > max_cross) { max_cross = dh[k]; jc = k; } }
                    else if (dh[k] > max_diag) { max_diag = dh[k]; jd = k; }
                }
            }
            if (bk > 0.0f) {
                const float sd = max_diag / SQRT2_F;
                const float slope = fmaxf(max_cross, sd);
                const int js = (jd >= 0 && sd > max_cross) ? jd : jc;
                const float alph = poly_atanf(slope);
                float s1 = 1.0f;
                const float newsh = 1.0f + alph - c.Kalpha0;
                const bool taken = newsh > s1;
                if (taken) s1 = newsh;
                const float sh3 = s1 * (s1 * s1);
                const float S = c.dt * c.Kspeed0 * sh3 * H / 2.0f;
                // reverse
                const float ac = as[si];
                const float rbk = __frcp_rn(bk);
                float g[8], gbar = 0.0f;
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    g[k] = mk[k] ? as[si + tt_oy(k) * TT_RW + tt_ox(k)] - ac : 0.0f;
                    gbar += g[k] * dh[k];
                }
                gbar *= rbk;
                const float sb = S * rbk;
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    if (mk[k]) gdh[k] = sb * (g[k] - gbar);
                const float dH = gbar * (c.dt * c.Kspeed0 * sh3 * 0.5f);
                if (taken && js >= 0) {
                    const float ds1 = gbar * (c.dt * c.Kspeed0 * H * 0.5f) * 3.0f * s1 * s1;
                    const float dslope = ds1 * __frcp_rn(1.0f + slope * slope);
#pragma unroll
                    for (int k = 0; k < 8; ++k)  // static indices keep gdh in registers
                        if (k == js) gdh[k] += k < 4 ? dslope : dslope * RCP_SQRT2_F;
                }
                if (Hmax < b) {
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        if (k == jh) gdh[k] += dH;
                } else {
                    own += dH;
                }
#pragma unroll
                for (int k = 0; k < 8; ++k) own += gdh[k];
            }
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) gd[k * TT_NC + q] = gdh[k];
        gd[8 * TT_NC + q] = own;
    }
    __syncthreads();
    // G(c) = A(c) + own(c) - sum over neighbours m of m's dL/ddh toward c
#pragma unroll 1
    for (int q = tid; q < TW * TT_H; q += TT_NTH) {
        const int ix = q % TW, iy = q / TW;
        const int x = tx0 + ix, y = ty0 + iy;
        const int rq = (iy + 1) * TT_CW + ix + 1;
        float gsum = as[(iy + 2) * TT_RW + HX + ix] + gd[8 * TT_NC + rq];  // A(c), from the staged box
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int xx = x + tt_ox(k), yy = y + tt_oy(k);
            if (EDGE && (xx < 0 || xx >= n || yy < 0 || yy >= n)) continue;
            gsum -= gd[(k ^ (k < 4 ? 1 : 3)) * TT_NC + rq + tt_oy(k) * TT_CW + tt_ox(k)];  // opposite direction
        }
        ta.g[(size_t)y * n + x] = gsum;
    }
}

constexpr size_t TT_SMEM = (2 * TT_BRC + 9 * TT_NC) * sizeof(float) + 8;

__global__ void __launch_bounds__(TT_NTH) k_adj_thermal(const __grid_constant__ ThermalArgs ta, int* err) {
    extern __shared__ __align__(128) float tdyn[];
    float* bs = tdyn;
    float* as = tdyn + TT_BRC;
    float* gd = tdyn + 2 * TT_BRC;
    uint64_t& bar = *reinterpret_cast<uint64_t*>(tdyn + 2 * TT_BRC + 9 * TT_NC);
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    const int n = ta.c.n;
    const int tiles_x = n / TW;
    const int tx0 = (blockIdx.x % tiles_x) * TW, ty0 = (blockIdx.x / tiles_x) * TT_H;
    bool inner = tx0 - HX >= 0 && tx0 + TW + HX <= n && ty0 - 2 >= 0 && ty0 + TT_H + 2 <= n;
    if (inner) thermal_tile<false>(ta, bs, as, gd, &bar, tx0, ty0, err);
    else thermal_tile<true>(ta, bs, as, gd, &bar, tx0, ty0, err);
}

// d(mean((rock - target)^2))/d rock, and the loss partials
__global__ void k_mse_grad(const float* __restrict__ b, const float* __restrict__ target, size_t count,
                           float* __restrict__ grad, double* __restrict__ part) {
    __shared__ double sh[256 / 32];
    double acc = 0.0;
    const double inv = 1.0 / (double)count;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        float e = b[i] - target[i];
        acc += (double)e * (double)e;
        if (grad) grad[i] = (float)(2.0 * (double)e * inv);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
        part[blockIdx.x] = t * inv;
    }
}

__global__ void k_sum_parts(const double* __restrict__ part, int nparts, double* __restrict__ out) {
    if (threadIdx.x != 0) return;
    double t = 0.0;
    for (int k = 0; k < nparts; ++k) t += part[k];
    *out = t;
}

// per-block sums of g^2 in FP64 (the gradient norm's accumulation)
__global__ void k_sumsq_part(const float* __restrict__ g, size_t count, double* __restrict__ part) {
    __shared__ double sh[256 / 32];
    double acc = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        acc += (double)g[i] * (double)g[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
        part[blockIdx.x] = t;
    }
}

// *out += sum of the partials (fixed order)
__global__ void k_add_parts(const double* __restrict__ part, int nparts, double* __restrict__ out) {
    if (threadIdx.x != 0) return;
    double t = 0.0;
    for (int k = 0; k < nparts; ++k) t += part[k];
    *out += t;
}

// per-block max |g| (max is order-free, so the result does not depend on the split)
__global__ void k_absmax_part(const float* __restrict__ g, size_t count, float* __restrict__ part) {
    __shared__ float sh[256 / 32];
    float m = 0.0f;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(g[i]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t = fmaxf(t, sh[k]);
        part[blockIdx.x] = t;
    }
}

// x <- clamp(x - (step / max|g|) g, lo, hi): the largest change of any cell is `step`
__global__ void k_descend(float* __restrict__ x, const float* __restrict__ g, size_t count,
                          const float* __restrict__ part, int nparts, float step, float lo, float hi) {
    __shared__ float a_sh;
    if (threadIdx.x < 32) {
        float m = 0.0f;
        for (int k = threadIdx.x; k < nparts; k += 32) m = fmaxf(m, part[k]);
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) a_sh = step / fmaxf(m, 1e-30f);
    }
    __syncthreads();
    const float a = a_sh;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        x[i] = fminf(fmaxf(x[i] - a * g[i], lo), hi);
}

dim3 grid_for(int n) { return dim3((n + BX - 1) / BX, (n + BY - 1) / BY); }

}  // namespace

bool adjoint_tile_ok(int n) { return n % TW == 0 && n % TH == 0; }

int adjoint_box_rows() { return H_RH; }

void launch_adjoint_sediment(const StepConsts& c, const AdjSlot& slot, const float* as, float* dse, float* du,
                             float* dv, cudaStream_t st) {
    k_adj_sediment<<<grid_for(c.n), dim3(BX, BY), 0, st>>>(c, slot, as, dse, du, dv);
    count_launch();
}

void launch_adjoint_cell(const AdjCellArgs& args, int* err, cudaStream_t st) {
    const int n = args.c.n;
    k_adj_cell<<<(n / TW) * (n / TH), NTH, 0, st>>>(args, err);
    count_launch();
}

void launch_adjoint_final(int n, const AdjView& A, float* out_b, cudaStream_t st) {
    k_adj_final<<<grid_for(n), dim3(BX, BY), 0, st>>>(n, A, out_b);
    count_launch();
}

int adjoint_thermal_box_rows() { return TT_BH; }

void launch_adjoint_thermal(const StepConsts& c, const CUtensorMap& map_b, const AdjView& A, float* g, int* err,
                            cudaStream_t st) {
    ThermalArgs ta;
    ta.map_b = map_b;
    ta.A = A;
    ta.c = c;
    ta.g = g;
    cudaFuncSetAttribute(k_adj_thermal, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TT_SMEM);
    k_adj_thermal<<<(c.n / TW) * (c.n / TT_H), TT_NTH, TT_SMEM, st>>>(ta, err);
    count_launch();
}

void launch_mse(const float* b, const float* target, size_t count, float* grad, double* part, int nparts,
                double* out, cudaStream_t st) {
    k_mse_grad<<<nparts, 256, 0, st>>>(b, target, count, grad, part);
    k_sum_parts<<<1, 32, 0, st>>>(part, nparts, out);
    count_launch(2);
}

void launch_add_sumsq(const float* g, size_t count, double* part, int nparts, double* out, cudaStream_t st) {
    k_sumsq_part<<<nparts, 256, 0, st>>>(g, count, part);
    k_add_parts<<<1, 32, 0, st>>>(part, nparts, out);
    count_launch(2);
}

void launch_descend(float* x, const float* g, size_t count, float step, float lo, float hi, float* part, int nparts,
                    cudaStream_t st) {
    k_absmax_part<<<nparts, 256, 0, st>>>(g, count, part);
    k_descend<<<nparts * 4, 256, 0, st>>>(x, g, count, part, nparts, step, lo, hi);
    count_launch(2);
}

}  // namespace hg
