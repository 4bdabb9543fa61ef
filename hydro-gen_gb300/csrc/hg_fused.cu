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
// any tap straight from HBM/L2.  The split costs 16 B per cell-step of
// intermediate traffic (eroded rock and sediment written and read once) and
// saves recomputing flux and erosion on a halo ring.
//
// k_hydro stages the tile's rock, water (+ this step's rain), and the four
// fluxes with a 1-cell halo (4 columns for 16-byte rows) in shared memory:
// one Philox call per four cells, coalesced float4 rows, then each thread
// computes four cells.  k_transport stages eroded rock with a 2-cell halo,
// computes each cell's eight talus outflows once (ring included) into shared
// memory, then applies outflow and inflow and the sediment gather.
//
// Per-cell arithmetic is the code of the per-pass kernels (hg_device.cuh),
// so the fused step reproduces them bit for bit.
#include "hg_internal.h"

namespace hg {

namespace {

constexpr int TW = 64, TH = 16, NTH = 256;
constexpr int CPT = TW * TH / NTH;  // cells per thread (4)
constexpr int HX = 4;               // halo columns: 16-byte aligned rows

__constant__ int f_ox[8] = {-1, 1, 0, 0, -1, 1, -1, 1};
__constant__ int f_oy[8] = {0, 0, 1, -1, 1, 1, -1, -1};
// direction from a neighbour back to this cell: L<->R, T<->B, LT<->RB, RT<->LB
__constant__ int f_opp[8] = {1, 0, 3, 2, 7, 6, 5, 4};

// ---------------------------------------------------------------------------
// k_hydro
// ---------------------------------------------------------------------------
constexpr int H_RW = TW + 2 * HX, H_RH = TH + 2, H_RC = H_RW * H_RH;
enum { H_B = 0, H_D, H_FL, H_FR, H_FT, H_FB, H_N };

template <bool EDGE>
__device__ __forceinline__ void hydro_tile(const FusedArgs& a, float* sm, int tx0, int ty0) {
    const StepConsts& c = a.c;
    const RainStep& r = a.rain[0];
    const int n = c.n;
    const int tid = threadIdx.x;
    const int gx0 = tx0 - HX, gy0 = ty0 - 1;
    const float* src[H_N] = {a.in.f[S_ROCK], a.in.f[S_WATER], a.in.f[S_FL], a.in.f[S_FR], a.in.f[S_FT],
                             a.in.f[S_FB]};
    constexpr int G4 = H_RW / 4;
    for (int q = tid; q < G4 * H_RH; q += NTH) {
        int ry = q / G4, rx = (q % G4) * 4;
        int gx = gx0 + rx, gy = gy0 + ry;
        bool ok = !EDGE || (gx >= 0 && gx < n && gy >= 0 && gy < n);
        size_t gi = (size_t)gy * n + gx;
        int si = ry * H_RW + rx;
#pragma unroll
        for (int f = 0; f < H_N; ++f) {
            float4 v = ok ? __ldg(reinterpret_cast<const float4*>(src[f] + gi)) : make_float4(0, 0, 0, 0);
            if (f == H_D && ok && r.active) {
                uint32_t w[4] = {0, 0, 0, 0};
                if (r.bernoulli) rain_words4(r, gx, gy, w);
                v.x += rain_incr(r, w[0]);
                v.y += rain_incr(r, w[1]);
                v.z += rain_incr(r, w[2]);
                v.w += rain_incr(r, w[3]);
            }
            *reinterpret_cast<float4*>(sm + f * H_RC + si) = v;
        }
    }
    __syncthreads();
    const float* B = sm + H_B * H_RC;
    const float* D = sm + H_D * H_RC;
    const float* FL = sm + H_FL * H_RC;
    const float* FR = sm + H_FR * H_RC;
    const float* FT = sm + H_FT * H_RC;
    const float* FB = sm + H_FB * H_RC;
#pragma unroll 1
    for (int k = 0; k < CPT; ++k) {
        int q = tid + k * NTH;
        int rx = HX + q % TW, ry = 1 + q / TW;
        int gx = gx0 + rx, gy = gy0 + ry;
        int si = ry * H_RW + rx;
        size_t gi = (size_t)gy * n + gx;
        auto tot = [&](int dx, int dy) -> float {
            if (EDGE) {
                int xx = gx + dx, yy = gy + dy;
                if (xx < 0 || xx >= n || yy < 0 || yy >= n) return FAR_HEIGHT;
            }
            int j = si + dy * H_RW + dx;
            return B[j] + D[j];
        };
        float d1 = D[si];
        float b = B[si];
        float w_c = b + d1;
        float inl = (!EDGE || gx > 0) ? FR[si - 1] : 0.0f;
        float inr = (!EDGE || gx < n - 1) ? FL[si + 1] : 0.0f;
        float int_ = (!EDGE || gy < n - 1) ? FB[si + H_RW] : 0.0f;
        float inb = (!EDGE || gy > 0) ? FT[si - H_RW] : 0.0f;
        FluxOut o = cell_flux(c, gx, gy, w_c, d1, FL[si], FR[si], FT[si], FB[si], tot(-1, 0), tot(1, 0), tot(0, 1),
                              tot(0, -1), inl, inr, int_, inb, EDGE);
        float s = __ldg(a.in.f[S_SED] + gi);
        float br = (!EDGE || gx < n - 1) ? B[si + 1] : 0.0f;
        float bl = (!EDGE || gx > 0) ? B[si - 1] : 0.0f;
        float bb = (!EDGE || gy > 0) ? B[si - H_RW] : 0.0f;
        float bt = (!EDGE || gy < n - 1) ? B[si + H_RW] : 0.0f;
        float Kls0 = c.ks_field ? c.dt * __ldg(c.ks_field + gi) : c.Kls0;
        cell_erosion(c, Kls0, o.u, o.v, o.vz, b, s, br, bl, bb, bt);
        a.out.f[S_FL][gi] = o.fl;
        a.out.f[S_FR][gi] = o.fr;
        a.out.f[S_FT][gi] = o.ft;
        a.out.f[S_FB][gi] = o.fb;
        a.out.f[S_WATER][gi] = o.d2 * c.evap;  // sediment_transport's evaporation (:75)
        a.u[gi] = o.u;
        a.v[gi] = o.v;
        a.s_ero[gi] = s;
        if (c.thermal) a.b_ero[gi] = b;
        else a.out.f[S_ROCK][gi] = b;  // no thermal pass: eroded rock is final
    }
}

__global__ void __launch_bounds__(NTH) k_hydro(FusedArgs a) {
    __shared__ __align__(16) float sm[H_N * H_RC];
    const int n = a.c.n;
    const int tx0 = blockIdx.x * TW, ty0 = blockIdx.y * TH;
    bool inner = tx0 - HX >= 0 && tx0 + TW + HX <= n && ty0 - 1 >= 0 && ty0 + TH + 1 <= n;
    if (inner) hydro_tile<false>(a, sm, tx0, ty0);
    else hydro_tile<true>(a, sm, tx0, ty0);
}

// ---------------------------------------------------------------------------
// k_transport
// ---------------------------------------------------------------------------
constexpr int T_RW = TW + 2 * HX, T_RH = TH + 4, T_RC = T_RW * T_RH;
// outflows are kept for interior plus 1: (TW + 2) x (TH + 2) cells
constexpr int O_W = TW + 2, O_H = TH + 2, O_C = O_W * O_H;

template <bool EDGE>
__device__ __forceinline__ void transport_tile(const FusedArgs& a, float* be, float* outf, int tx0, int ty0) {
    const StepConsts& c = a.c;
    const int n = c.n;
    const int tid = threadIdx.x;
    const int gx0 = tx0 - HX, gy0 = ty0 - 2;
    if (c.thermal) {
        constexpr int G4 = T_RW / 4;
        for (int q = tid; q < G4 * T_RH; q += NTH) {
            int ry = q / G4, rx = (q % G4) * 4;
            int gx = gx0 + rx, gy = gy0 + ry;
            bool ok = !EDGE || (gx >= 0 && gx < n && gy >= 0 && gy < n);
            float4 v = ok ? __ldg(reinterpret_cast<const float4*>(a.b_ero + (size_t)gy * n + gx))
                          : make_float4(0, 0, 0, 0);
            *reinterpret_cast<float4*>(be + ry * T_RW + rx) = v;
        }
        __syncthreads();
        // eight outflows of every cell of interior plus 1 (the shader's
        // thermal_erosion pass), each directed edge's division done once
        for (int q = tid; q < O_C; q += NTH) {
            int ox = q % O_W, oy = q / O_W;
            int rx = HX - 1 + ox, ry = 1 + oy;
            int gx = gx0 + rx, gy = gy0 + ry;
            float o8[8];
            if (EDGE && (gx < 0 || gx >= n || gy < 0 || gy >= n)) {
#pragma unroll
                for (int d = 0; d < 8; ++d) o8[d] = 0.0f;
            } else {
                int si = ry * T_RW + rx;
                float b = be[si];
                float nb[8];
#pragma unroll
                for (int d = 0; d < 8; ++d) {
                    bool out = false;
                    if (EDGE) {
                        int xx = gx + f_ox[d], yy = gy + f_oy[d];
                        out = xx < 0 || xx >= n || yy < 0 || yy >= n;
                    }
                    nb[d] = out ? FAR_HEIGHT : be[si + f_oy[d] * T_RW + f_ox[d]];
                }
                ThermalOut t = cell_thermal_fast(c, b, nb);
#pragma unroll
                for (int d = 0; d < 8; ++d) o8[d] = (t.mask >> d & 1u) ? t.S * (b - nb[d]) / t.bk : 0.0f;
            }
#pragma unroll
            for (int d = 0; d < 8; ++d) outf[d * O_C + q] = o8[d];
        }
        __syncthreads();
    }
#pragma unroll 1
    for (int k = 0; k < CPT; ++k) {
        int q = tid + k * NTH;
        int ix0 = q % TW, iy0 = q / TW;
        int gx = tx0 + ix0, gy = ty0 + iy0;
        size_t gi = (size_t)gy * n + gx;
        // sediment_transport: semi-Lagrangian gather of eroded sediment
        float px, py;
        backtrace(c, gx, gy, __ldg(a.u + gi), __ldg(a.v + gi), px, py);
        int ix = min(max((int)px, 0), n - 1), iy = min(max((int)py, 0), n - 1);
        const float* se = a.s_ero + (size_t)iy * n + ix;
        float s00 = __ldg(se);
        float s10 = ix + 1 < n ? __ldg(se + 1) : 0.0f;
        float s01 = iy + 1 < n ? __ldg(se + n) : 0.0f;
        float s11 = (ix + 1 < n && iy + 1 < n) ? __ldg(se + n + 1) : 0.0f;
        a.out.f[S_SED][gi] = bilinear_mix(px, py, s00, s10, s01, s11);
        // thermal_transport: own outflows out, neighbours' outflows in
        if (c.thermal) {
            int oi = (iy0 + 1) * O_W + (ix0 + 1);
            float own[8], in[8];
#pragma unroll
            for (int d = 0; d < 8; ++d) {
                own[d] = outf[d * O_C + oi];
                in[d] = outf[f_opp[d] * O_C + oi + f_oy[d] * O_W + f_ox[d]];
            }
            float b = be[(iy0 + 2) * T_RW + ix0 + HX];
            a.out.f[S_ROCK][gi] = cell_thermal_apply(b, own, in);
        }
    }
}

__global__ void __launch_bounds__(NTH) k_transport(FusedArgs a) {
    __shared__ __align__(16) float be[T_RC];
    __shared__ float outf[8 * O_C];
    const int n = a.c.n;
    const int tx0 = blockIdx.x * TW, ty0 = blockIdx.y * TH;
    bool inner = tx0 - HX >= 0 && tx0 + TW + HX <= n && ty0 - 2 >= 0 && ty0 + TH + 2 <= n;
    if (inner) transport_tile<false>(a, be, outf, tx0, ty0);
    else transport_tile<true>(a, be, outf, tx0, ty0);
}

}  // namespace

int fused_max_depth() { return 1; }

bool fused_supported(int depth, int tile_x, int tile_y) { return depth == 1 && tile_x == TW && tile_y == TH; }

void launch_fused(const FusedArgs& a, int depth, int tile_x, int tile_y, cudaStream_t st) {
    (void)depth; (void)tile_x; (void)tile_y;
    dim3 grid(a.c.n / TW, a.c.n / TH);
    k_hydro<<<grid, NTH, 0, st>>>(a);
    k_transport<<<grid, NTH, 0, st>>>(a);
    count_launch(2);
}

}  // namespace hg
