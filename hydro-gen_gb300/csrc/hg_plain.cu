// Per-pass kernels: one kernel per GLSL pass of the grid step, FP32
// structure-of-arrays fields, one cell per thread (rows of 32 cells per warp,
// so every field access of a warp is a 128-byte coalesced line), Jacobi
// ping-pong between passes as in the reference (src/erosion.cpp:158-200).
#include "hg_internal.h"

namespace hg {

namespace {

constexpr int BX = 32, BY = 8;

__device__ __forceinline__ size_t at(int n, int x, int y) { return (size_t)y * n + x; }

// glsl/rain.glsl:32-56 — four cells per thread share one Philox call.
__global__ void k_rain(StepConsts c, RainStep r, float* __restrict__ water) {
    int x0 = (blockIdx.x * blockDim.x + threadIdx.x) * 4;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x0 >= c.n || y < c.row_lo || y >= c.row_hi) return;
    float4* p = reinterpret_cast<float4*>(water + at(c.n, x0, y));
    float4 d = *p;
    uint32_t w[4] = {0, 0, 0, 0};
    if (r.bernoulli) rain_words4(r, x0, y, w);
    d.x += rain_incr(r, w[0]);
    d.y += rain_incr(r, w[1]);
    d.z += rain_incr(r, w[2]);
    d.w += rain_incr(r, w[3]);
    *p = d;
}

// glsl/hydro_flux.glsl:77-166
__global__ void k_flux(StepConsts c, const float* __restrict__ rock, const float* __restrict__ water,
                       const float* __restrict__ fl, const float* __restrict__ fr,
                       const float* __restrict__ ft, const float* __restrict__ fb,
                       float* __restrict__ water_o, float* __restrict__ fl_o, float* __restrict__ fr_o,
                       float* __restrict__ ft_o, float* __restrict__ fb_o, float* __restrict__ u_o,
                       float* __restrict__ v_o, float* __restrict__ vz_o) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y < c.row_lo || y >= c.row_hi) return;
    size_t i = at(n, x, y);
    auto total = [&](int xx, int yy) -> float {
        if (xx < 0 || xx >= n || yy < 0 || yy >= n) return FAR_HEIGHT;
        size_t j = at(n, xx, yy);
        return rock[j] + water[j];
    };
    float d1 = water[i];
    float w_c = rock[i] + d1;
    float inl = x > 0 ? fr[i - 1] : 0.0f;
    float inr = x < n - 1 ? fl[i + 1] : 0.0f;
    float int_ = y < n - 1 ? fb[i + n] : 0.0f;
    float inb = y > 0 ? ft[i - n] : 0.0f;
    FluxOut o = cell_flux(c, x, y, w_c, d1, fl[i], fr[i], ft[i], fb[i], total(x - 1, y), total(x + 1, y),
                          total(x, y + 1), total(x, y - 1), inl, inr, int_, inb);
    fl_o[i] = o.fl; fr_o[i] = o.fr; ft_o[i] = o.ft; fb_o[i] = o.fb;
    water_o[i] = o.d2;
    u_o[i] = o.u; v_o[i] = o.v; vz_o[i] = o.vz;
}

// glsl/hydro_erosion.glsl:37-92
__global__ void k_erosion(StepConsts c, const float* __restrict__ u, const float* __restrict__ v,
                          const float* __restrict__ vz, const float* __restrict__ rock,
                          float* __restrict__ rock_o, float* __restrict__ sed) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y < c.row_lo || y >= c.row_hi) return;
    size_t i = at(n, x, y);
    float br = x < n - 1 ? rock[i + 1] : 0.0f;
    float bl = x > 0 ? rock[i - 1] : 0.0f;
    float bb = y > 0 ? rock[i - n] : 0.0f;
    float bt = y < n - 1 ? rock[i + n] : 0.0f;
    float b = rock[i], s = sed[i];
    float Kls0 = c.ks_field ? c.dt * c.ks_field[i] : c.Kls0;
    cell_erosion(c, Kls0, u[i], v[i], vz[i], b, s, br, bl, bb, bt);
    rock_o[i] = b;
    sed[i] = s;
}

// glsl/sediment_transport.glsl:66-93
__global__ void k_sediment(StepConsts c, const float* __restrict__ u, const float* __restrict__ v,
                           const float* __restrict__ sed, float* __restrict__ sed_o,
                           float* __restrict__ water) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y < c.row_lo || y >= c.row_hi) return;
    size_t i = at(n, x, y);
    float px, py;
    backtrace(c, x, y, u[i], v[i], px, py);
    int ix = (int)px, iy = (int)py;
    auto tap = [&](int xx, int yy) -> float {
        return (xx >= 0 && xx < n && yy >= 0 && yy < n) ? sed[at(n, xx, yy)] : 0.0f;
    };
    sed_o[i] = bilinear_mix(px, py, tap(ix, iy), tap(ix + 1, iy), tap(ix, iy + 1), tap(ix + 1, iy + 1));
    water[i] = water[i] * c.evap;
}

__constant__ int c_ox[8] = {-1, 1, 0, 0, -1, 1, -1, 1};
__constant__ int c_oy[8] = {0, 0, 1, -1, 1, 1, -1, -1};

// glsl/thermal_erosion.glsl:28-115, layer 0
__global__ void k_thermal_out(StepConsts c, const float* __restrict__ rock, float4* __restrict__ tc,
                              float4* __restrict__ td) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y < c.row_lo || y >= c.row_hi) return;
    size_t i = at(n, x, y);
    float b = rock[i];
    float nb[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        int xx = x + c_ox[k], yy = y + c_oy[k];
        nb[k] = (xx < 0 || xx >= n || yy < 0 || yy >= n) ? FAR_HEIGHT : rock[at(n, xx, yy)];
    }
    ThermalOut t = cell_thermal_ref(c, b, nb);
    float o[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) o[k] = (t.mask >> k & 1u) ? t.S * (b - nb[k]) / t.bk : 0.0f;
    tc[i] = make_float4(o[0], o[1], o[2], o[3]);
    td[i] = make_float4(o[4], o[5], o[6], o[7]);
}

// glsl/thermal_transport.glsl:31-65, layer 0
__global__ void k_thermal_in(StepConsts c, const float* __restrict__ rock, const float4* __restrict__ tc,
                             const float4* __restrict__ td, float* __restrict__ rock_o) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y < c.row_lo || y >= c.row_hi) return;
    size_t i = at(n, x, y);
    auto ok = [&](int xx, int yy) { return xx >= 0 && xx < n && yy >= 0 && yy < n; };
    float in[8];
    in[0] = ok(x - 1, y) ? tc[i - 1].y : 0.0f;
    in[1] = ok(x + 1, y) ? tc[i + 1].x : 0.0f;
    in[2] = ok(x, y + 1) ? tc[i + n].w : 0.0f;
    in[3] = ok(x, y - 1) ? tc[i - n].z : 0.0f;
    in[4] = ok(x - 1, y + 1) ? td[i + n - 1].w : 0.0f;
    in[5] = ok(x + 1, y + 1) ? td[i + n + 1].z : 0.0f;
    in[6] = ok(x - 1, y - 1) ? td[i - n - 1].y : 0.0f;
    in[7] = ok(x + 1, y - 1) ? td[i - n + 1].x : 0.0f;
    float4 a = tc[i], b4 = td[i];
    float own[8] = {a.x, a.y, a.z, a.w, b4.x, b4.y, b4.z, b4.w};
    rock_o[i] = cell_thermal_apply(rock[i], own, in);
}

// glsl/smoothing.glsl:22-103, rock channel (see cell_smooth)
__global__ void k_smooth(StepConsts c, const float* __restrict__ rock, float* __restrict__ rock_o) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y < c.row_lo || y >= c.row_hi) return;
    size_t i = at(n, x, y);
    if (x == 0 || y == 0 || x == n - 1 || y == n - 1) {  // border texels are copied (:27-33)
        rock_o[i] = rock[i];
        return;
    }
    rock_o[i] = cell_smooth(c.smooth_m, rock[i], rock[i - 1], rock[i + 1], rock[i + n], rock[i - n]);
}

dim3 grid_for(int n) { return dim3((n + BX - 1) / BX, (n + BY - 1) / BY); }

}  // namespace

void launch_rain(const StepConsts& c, const RainStep& r, float* water, cudaStream_t st) {
    dim3 blk(BX, BY), grd((c.n / 4 + BX - 1) / BX, (c.n + BY - 1) / BY);
    k_rain<<<grd, blk, 0, st>>>(c, r, water);
    count_launch();
}

void launch_flux(const StepConsts& c, const float* rock, const float* water, const float* fl, const float* fr,
                 const float* ft, const float* fb, float* water_o, float* fl_o, float* fr_o, float* ft_o,
                 float* fb_o, float* u, float* v, float* vz, cudaStream_t st) {
    k_flux<<<grid_for(c.n), dim3(BX, BY), 0, st>>>(c, rock, water, fl, fr, ft, fb, water_o, fl_o, fr_o, ft_o,
                                                   fb_o, u, v, vz);
    count_launch();
}

void launch_erosion(const StepConsts& c, const float* u, const float* v, const float* vz, const float* rock,
                    float* rock_o, float* sed_inout, cudaStream_t st) {
    k_erosion<<<grid_for(c.n), dim3(BX, BY), 0, st>>>(c, u, v, vz, rock, rock_o, sed_inout);
    count_launch();
}

void launch_sediment(const StepConsts& c, const float* u, const float* v, const float* sed, float* sed_o,
                     float* water_inout, cudaStream_t st) {
    k_sediment<<<grid_for(c.n), dim3(BX, BY), 0, st>>>(c, u, v, sed, sed_o, water_inout);
    count_launch();
}

void launch_thermal_out(const StepConsts& c, const float* rock, float4* tc, float4* td, cudaStream_t st) {
    k_thermal_out<<<grid_for(c.n), dim3(BX, BY), 0, st>>>(c, rock, tc, td);
    count_launch();
}

void launch_thermal_in(const StepConsts& c, const float* rock, const float4* tc, const float4* td,
                       float* rock_o, cudaStream_t st) {
    k_thermal_in<<<grid_for(c.n), dim3(BX, BY), 0, st>>>(c, rock, tc, td, rock_o);
    count_launch();
}

void launch_smooth(const StepConsts& c, const float* rock, float* rock_o, cudaStream_t st) {
    k_smooth<<<grid_for(c.n), dim3(BX, BY), 0, st>>>(c, rock, rock_o);
    count_launch();
}

}  // namespace hg
