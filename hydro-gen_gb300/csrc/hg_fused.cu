// Fused grid step: rain -> hydro_flux -> hydro_erosion -> sediment_transport
// -> thermal (layer 0) for a whole step in one persistent kernel.
//
// Each CTA walks a list of TW x TH output tiles.  For a tile it stages the
// carried fields (rock, water, sediment, four fluxes) of the tile plus a halo
// (HX columns, HY rows on each side) in shared memory, then runs the passes
// over shrinking sub-rectangles of the staged region:
//   load (+rain)           region
//   A: flux + erosion       region minus 1   -> eroded rock, eroded sediment,
//                                              u, v in shared memory; new
//                                              flux and evaporated water of
//                                              interior cells go straight out
//   B: thermal outflow      region minus 2   -> S, bk, direction mask
//   C: sediment + thermal   tile interior    -> rock, sediment out
// The per-cell arithmetic is the same code as the per-pass kernels
// (hg_device.cuh), so the fused step reproduces them bit for bit.
//
// The semi-Lagrangian back-trace reach |u|*dt is data dependent.  A tap that
// lands outside the staged region is recomputed from the step's input
// fields in global memory (s_ero_global), so results never depend on the
// halo width.
#include "hg_internal.h"

namespace hg {

namespace {

constexpr int HX = 4;  // halo columns (multiple of 4: float4 row staging)
constexpr int HY = 3;  // halo rows: erosion 1 + thermal 2
constexpr int NARR = 10;
enum { A_B = 0, A_D, A_S, A_FL, A_FR, A_FT, A_FB, A_B2, A_U, A_V };
// thermal exchange reuses the flux arrays once pass A is done
constexpr int A_TS = A_FL, A_TBK = A_FR, A_TMASK = A_FT;

__constant__ int f_ox[8] = {-1, 1, 0, 0, -1, 1, -1, 1};
__constant__ int f_oy[8] = {0, 0, 1, -1, 1, 1, -1, -1};
// direction from a neighbour back to this cell: L<->R, T<->B, LT<->RB, RT<->LB
__constant__ int f_opp[8] = {1, 0, 3, 2, 7, 6, 5, 4};

struct Ctx {
    const FusedArgs* a;
    int n;
};

// Rain increment of cell (x, y) for one step (recomputes the Philox group).
__device__ __forceinline__ float rain_at(const RainStep& r, int x, int y) {
    if (!r.active) return 0.0f;
    uint32_t w[4] = {0, 0, 0, 0};
    if (r.bernoulli) rain_words4(r, x & ~3, y, w);
    return rain_incr(r, w[x & 3]);
}

// Eroded sediment of cell (tx, ty) of the current step, computed from the
// step's input fields in global memory (rain, flux and erosion of one cell).
__device__ float s_ero_global(const FusedArgs& a, const RainStep& r, int tx, int ty) {
    const StepConsts& c = a.c;
    const int n = c.n;
    const float* rock = a.in.f[S_ROCK];
    const float* water = a.in.f[S_WATER];
    auto idx = [&](int x, int y) { return (size_t)y * n + x; };
    auto inside = [&](int x, int y) { return x >= 0 && x < n && y >= 0 && y < n; };
    auto total = [&](int x, int y) -> float {
        if (!inside(x, y)) return FAR_HEIGHT;
        return rock[idx(x, y)] + (water[idx(x, y)] + rain_at(r, x, y));
    };
    size_t i = idx(tx, ty);
    float d1 = water[i] + rain_at(r, tx, ty);
    float w_c = rock[i] + d1;
    float inl = tx > 0 ? a.in.f[S_FR][i - 1] : 0.0f;
    float inr = tx < n - 1 ? a.in.f[S_FL][i + 1] : 0.0f;
    float int_ = ty < n - 1 ? a.in.f[S_FB][i + n] : 0.0f;
    float inb = ty > 0 ? a.in.f[S_FT][i - n] : 0.0f;
    FluxOut o = cell_flux(c, tx, ty, w_c, d1, a.in.f[S_FL][i], a.in.f[S_FR][i], a.in.f[S_FT][i], a.in.f[S_FB][i],
                          total(tx - 1, ty), total(tx + 1, ty), total(tx, ty + 1), total(tx, ty - 1), inl, inr,
                          int_, inb);
    float b = rock[i], s = a.in.f[S_SED][i];
    float br = tx < n - 1 ? rock[i + 1] : 0.0f;
    float bl = tx > 0 ? rock[i - 1] : 0.0f;
    float bb = ty > 0 ? rock[i - n] : 0.0f;
    float bt = ty < n - 1 ? rock[i + n] : 0.0f;
    float Kls0 = c.ks_field ? c.dt * c.ks_field[i] : c.Kls0;
    cell_erosion(c, Kls0, o.u, o.v, o.vz, b, s, br, bl, bb, bt);
    return s;
}

template <int TW, int TH>
__global__ void __launch_bounds__(256) k_fused(FusedArgs a) {
    constexpr int RW = TW + 2 * HX, RH = TH + 2 * HY, RC = RW * RH;
    extern __shared__ float smem[];
    float* arr[NARR];
#pragma unroll
    for (int k = 0; k < NARR; ++k) arr[k] = smem + k * RC;
    const StepConsts& c = a.c;
    const RainStep& r = a.rain[0];
    const int n = c.n;
    const int tiles_x = n / TW, tiles_y = n / TH, ntiles = tiles_x * tiles_y;
    const int tid = threadIdx.x, nth = blockDim.x;

    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int tx0 = (tile % tiles_x) * TW, ty0 = (tile / tiles_x) * TH;
        const int gx0 = tx0 - HX, gy0 = ty0 - HY;  // global coords of region (0, 0)

        // ---- stage the region (float4 groups never straddle the grid edge) ----
        constexpr int G4 = RW / 4;
        for (int q = tid; q < G4 * RH; q += nth) {
            int ry = q / G4, rx = (q % G4) * 4;
            int gx = gx0 + rx, gy = gy0 + ry;
            bool ok = gx >= 0 && gx < n && gy >= 0 && gy < n;
            size_t gi = (size_t)gy * n + gx;
            int si = ry * RW + rx;
#pragma unroll
            for (int f = 0; f < S_COUNT; ++f) {
                float4 v = ok ? __ldg(reinterpret_cast<const float4*>(a.in.f[f] + gi)) : make_float4(0, 0, 0, 0);
                if (f == S_WATER && ok && r.active) {
                    uint32_t w[4] = {0, 0, 0, 0};
                    if (r.bernoulli) rain_words4(r, gx, gy, w);
                    v.x += rain_incr(r, w[0]);
                    v.y += rain_incr(r, w[1]);
                    v.z += rain_incr(r, w[2]);
                    v.w += rain_incr(r, w[3]);
                }
                *reinterpret_cast<float4*>(arr[f] + si) = v;
            }
        }
        __syncthreads();

        // ---- A: flux + erosion on region minus 1 -------------------------------
        {
            constexpr int AW = RW - 2, AH = RH - 2;
            for (int q = tid; q < AW * AH; q += nth) {
                int rx = 1 + q % AW, ry = 1 + q / AW;
                int gx = gx0 + rx, gy = gy0 + ry;
                if (gx < 0 || gx >= n || gy < 0 || gy >= n) continue;
                int si = ry * RW + rx;
                auto tot = [&](int dx, int dy) -> float {
                    int xx = gx + dx, yy = gy + dy;
                    if (xx < 0 || xx >= n || yy < 0 || yy >= n) return FAR_HEIGHT;
                    int j = si + dy * RW + dx;
                    return arr[A_B][j] + arr[A_D][j];
                };
                float d1 = arr[A_D][si];
                float w_c = arr[A_B][si] + d1;
                float inl = gx > 0 ? arr[A_FR][si - 1] : 0.0f;
                float inr = gx < n - 1 ? arr[A_FL][si + 1] : 0.0f;
                float int_ = gy < n - 1 ? arr[A_FB][si + RW] : 0.0f;
                float inb = gy > 0 ? arr[A_FT][si - RW] : 0.0f;
                FluxOut o = cell_flux(c, gx, gy, w_c, d1, arr[A_FL][si], arr[A_FR][si], arr[A_FT][si],
                                      arr[A_FB][si], tot(-1, 0), tot(1, 0), tot(0, 1), tot(0, -1), inl, inr, int_,
                                      inb);
                float b = arr[A_B][si], s = arr[A_S][si];
                float br = gx < n - 1 ? arr[A_B][si + 1] : 0.0f;
                float bl = gx > 0 ? arr[A_B][si - 1] : 0.0f;
                float bb = gy > 0 ? arr[A_B][si - RW] : 0.0f;
                float bt = gy < n - 1 ? arr[A_B][si + RW] : 0.0f;
                size_t gi = (size_t)gy * n + gx;
                float Kls0 = c.ks_field ? c.dt * __ldg(c.ks_field + gi) : c.Kls0;
                cell_erosion(c, Kls0, o.u, o.v, o.vz, b, s, br, bl, bb, bt);
                arr[A_B2][si] = b;
                arr[A_S][si] = s;  // only this cell reads its own sediment in pass A
                arr[A_U][si] = o.u;
                arr[A_V][si] = o.v;
                bool interior = rx >= HX && rx < HX + TW && ry >= HY && ry < HY + TH;
                if (interior) {
                    a.out.f[S_FL][gi] = o.fl;
                    a.out.f[S_FR][gi] = o.fr;
                    a.out.f[S_FT][gi] = o.ft;
                    a.out.f[S_FB][gi] = o.fb;
                    a.out.f[S_WATER][gi] = o.d2 * c.evap;  // sediment pass evaporation
                    a.u[gi] = o.u;
                    a.v[gi] = o.v;
                }
            }
        }
        __syncthreads();

        // ---- B: thermal outflow on region minus 2 ------------------------------
        if (c.thermal) {
            constexpr int BW = RW - 4, BH = RH - 4;
            for (int q = tid; q < BW * BH; q += nth) {
                int rx = 2 + q % BW, ry = 2 + q / BW;
                int gx = gx0 + rx, gy = gy0 + ry;
                if (gx < 0 || gx >= n || gy < 0 || gy >= n) continue;
                int si = ry * RW + rx;
                float nb[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    int xx = gx + f_ox[k], yy = gy + f_oy[k];
                    nb[k] = (xx < 0 || xx >= n || yy < 0 || yy >= n) ? FAR_HEIGHT
                                                                       : arr[A_B2][si + f_oy[k] * RW + f_ox[k]];
                }
                ThermalOut t = cell_thermal_fast(c, arr[A_B2][si], nb);
                arr[A_TS][si] = t.S;
                arr[A_TBK][si] = t.bk;
                arr[A_TMASK][si] = __uint_as_float(t.mask);
            }
            __syncthreads();
        }

        // ---- C: sediment transport + thermal transport on the interior ----------
        for (int q = tid; q < TW * TH; q += nth) {
            int rx = HX + q % TW, ry = HY + q / TW;
            int gx = gx0 + rx, gy = gy0 + ry;
            int si = ry * RW + rx;
            size_t gi = (size_t)gy * n + gx;
            // sediment_transport: bilinear gather of eroded sediment
            float px, py;
            backtrace(c, gx, gy, arr[A_U][si], arr[A_V][si], px, py);
            int ix = min(max((int)px, 0), n - 1), iy = min(max((int)py, 0), n - 1);
            int lx = ix - gx0, ly = iy - gy0;  // region coords of the (ix, iy) tap
            float s00, s10, s01, s11;
            bool staged = lx >= 1 && lx + 1 <= RW - 2 && ly >= 1 && ly + 1 <= RH - 2;
            if (staged) {
                int j = ly * RW + lx;
                s00 = arr[A_S][j];
                s10 = ix + 1 < n ? arr[A_S][j + 1] : 0.0f;
                s01 = iy + 1 < n ? arr[A_S][j + RW] : 0.0f;
                s11 = (ix + 1 < n && iy + 1 < n) ? arr[A_S][j + RW + 1] : 0.0f;
            } else {
                s00 = s_ero_global(a, r, ix, iy);
                s10 = ix + 1 < n ? s_ero_global(a, r, ix + 1, iy) : 0.0f;
                s01 = iy + 1 < n ? s_ero_global(a, r, ix, iy + 1) : 0.0f;
                s11 = (ix + 1 < n && iy + 1 < n) ? s_ero_global(a, r, ix + 1, iy + 1) : 0.0f;
            }
            float s_new = bilinear_mix(px, py, s00, s10, s01, s11);
            // thermal_transport
            float b2 = arr[A_B2][si];
            float b_new = b2;
            if (c.thermal) {
                float S = arr[A_TS][si], bk = arr[A_TBK][si];
                uint32_t mask = __float_as_uint(arr[A_TMASK][si]);
                float own[8], in[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    int xx = gx + f_ox[k], yy = gy + f_oy[k];
                    bool ok = xx >= 0 && xx < n && yy >= 0 && yy < n;
                    int j = si + f_oy[k] * RW + f_ox[k];
                    float bn = ok ? arr[A_B2][j] : FAR_HEIGHT;
                    own[k] = (mask >> k & 1u) ? S * (b2 - bn) / bk : 0.0f;
                    in[k] = 0.0f;
                    if (ok) {
                        uint32_t m = __float_as_uint(arr[A_TMASK][j]);
                        if (m >> f_opp[k] & 1u) in[k] = arr[A_TS][j] * (bn - b2) / arr[A_TBK][j];
                    }
                }
                b_new = cell_thermal_apply(b2, own, in);
            }
            a.out.f[S_ROCK][gi] = b_new;
            a.out.f[S_SED][gi] = s_new;
        }
        __syncthreads();
    }
}

template <int TW, int TH>
size_t smem_bytes() {
    return sizeof(float) * NARR * (size_t)(TW + 2 * HX) * (TH + 2 * HY);
}

template <int TW, int TH>
void launch_tile(const FusedArgs& a, cudaStream_t st) {
    static int grid = 0;
    size_t sm = smem_bytes<TW, TH>();
    if (!grid) {
        cudaFuncSetAttribute(k_fused<TW, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        int dev = 0, nsm = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_fused<TW, TH>, 256, sm);
        grid = nsm * (per > 0 ? per : 1);
    }
    int ntiles = (a.c.n / TW) * (a.c.n / TH);
    k_fused<TW, TH><<<ntiles < grid ? ntiles : grid, 256, sm, st>>>(a);
    count_launch();
}

}  // namespace

int fused_max_depth() { return 1; }

bool fused_supported(int depth, int tile_x, int tile_y) {
    return depth == 1 && ((tile_x == 64 && tile_y == 32) || (tile_x == 32 && tile_y == 32) ||
                          (tile_x == 64 && tile_y == 16));
}

void launch_fused(const FusedArgs& a, int depth, int tile_x, int tile_y, cudaStream_t st) {
    (void)depth;
    if (tile_x == 64 && tile_y == 32) launch_tile<64, 32>(a, st);
    else if (tile_x == 32 && tile_y == 32) launch_tile<32, 32>(a, st);
    else launch_tile<64, 16>(a, st);
}

}  // namespace hg
