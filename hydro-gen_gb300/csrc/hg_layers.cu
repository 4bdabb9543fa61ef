// Per-pass kernels of the two-layer world (rock + dirt): the reference's
// full material model.  Rock sits in heightmap.r, dirt in heightmap.g, rock
// sediment in sedimap.r and dirt sediment in sedimap.g
// (glsl/heightmap.glsl:138-146, src/rendering.cpp:214); the total height the
// flux pass compares is (rock + dirt) + water, the order in which every pass
// before it leaves the total channel.  Rain reuses k_rain; thermal layer 0
// reuses k_thermal_out / k_thermal_in (its drops involve rock only).
#include "hg_internal.h"

namespace hg {

namespace {

constexpr int BX = 32, BY = 8;
__device__ __forceinline__ size_t at(int n, int x, int y) { return (size_t)y * n + x; }
__device__ __forceinline__ bool inside(int n, int x, int y) { return x >= 0 && x < n && y >= 0 && y < n; }

// glsl/hydro_flux.glsl:77-166 with the two-layer total
__global__ void k2_flux(StepConsts c, const float* __restrict__ rock, const float* __restrict__ dirt,
                        const float* __restrict__ water, const float* __restrict__ fl, const float* __restrict__ fr,
                        const float* __restrict__ ft, const float* __restrict__ fb, float* __restrict__ water_o,
                        float* __restrict__ fl_o, float* __restrict__ fr_o, float* __restrict__ ft_o,
                        float* __restrict__ fb_o, float* __restrict__ u_o, float* __restrict__ v_o,
                        float* __restrict__ vz_o) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y >= n) return;
    size_t i = at(n, x, y);
    auto total = [&](int xx, int yy) -> float {
        if (!inside(n, xx, yy)) return FAR_HEIGHT;
        size_t j = at(n, xx, yy);
        return rock[j] + dirt[j] + water[j];
    };
    float d1 = water[i];
    float inl = x > 0 ? fr[i - 1] : 0.0f;
    float inr = x < n - 1 ? fl[i + 1] : 0.0f;
    float int_ = y < n - 1 ? fb[i + n] : 0.0f;
    float inb = y > 0 ? ft[i - n] : 0.0f;
    FluxOut o = cell_flux(c, x, y, total(x, y), d1, fl[i], fr[i], ft[i], fb[i], total(x - 1, y), total(x + 1, y),
                          total(x, y + 1), total(x, y - 1), inl, inr, int_, inb);
    fl_o[i] = o.fl; fr_o[i] = o.fr; ft_o[i] = o.ft; fb_o[i] = o.fb;
    water_o[i] = o.d2;
    u_o[i] = o.u; v_o[i] = o.v; vz_o[i] = o.vz;
}

// glsl/hydro_erosion.glsl:23-92, both layers
__global__ void k2_erosion(StepConsts c, const float* __restrict__ u, const float* __restrict__ v,
                           const float* __restrict__ vz, const float* __restrict__ rock,
                           const float* __restrict__ dirt, float* __restrict__ rock_o, float* __restrict__ dirt_o,
                           float* __restrict__ s0, float* __restrict__ s1) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y >= n) return;
    size_t i = at(n, x, y);
    auto R = [&](int xx, int yy) { return inside(n, xx, yy) ? rock[at(n, xx, yy)] : 0.0f; };
    auto D = [&](int xx, int yy) { return inside(n, xx, yy) ? dirt[at(n, xx, yy)] : 0.0f; };
    float r = rock[i], g = dirt[i], a = s0[i], b = s1[i];
    float Kls0 = c.ks_field ? c.dt * c.ks_field[i] : c.Kls0;
    cell_erosion2(c, Kls0, u[i], v[i], vz[i], r, g, a, b, R(x + 1, y), D(x + 1, y), R(x - 1, y), D(x - 1, y),
                  R(x, y + 1), D(x, y + 1), R(x, y - 1), D(x, y - 1));
    rock_o[i] = r;
    dirt_o[i] = g;
    s0[i] = a;
    s1[i] = b;
}

// glsl/sediment_transport.glsl:66-93, both sediment channels
__global__ void k2_sediment(StepConsts c, const float* __restrict__ u, const float* __restrict__ v,
                            const float* __restrict__ s0, const float* __restrict__ s1, float* __restrict__ s0_o,
                            float* __restrict__ s1_o, float* __restrict__ water) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y >= n) return;
    size_t i = at(n, x, y);
    float px, py;
    backtrace(c, x, y, u[i], v[i], px, py);
    int ix = (int)px, iy = (int)py;
    auto tap = [&](const float* s, int xx, int yy) -> float { return inside(n, xx, yy) ? s[at(n, xx, yy)] : 0.0f; };
    s0_o[i] = bilinear_mix(px, py, tap(s0, ix, iy), tap(s0, ix + 1, iy), tap(s0, ix, iy + 1), tap(s0, ix + 1, iy + 1));
    s1_o[i] = bilinear_mix(px, py, tap(s1, ix, iy), tap(s1, ix + 1, iy), tap(s1, ix, iy + 1), tap(s1, ix + 1, iy + 1));
    water[i] = water[i] * c.evap;
}

__constant__ int c2_ox[8] = {-1, 1, 0, 0, -1, 1, -1, 1};
__constant__ int c2_oy[8] = {0, 0, 1, -1, 1, 1, -1, -1};

// glsl/thermal_erosion.glsl:28-109, layer 1: drops summed over rock and
// dirt ((0 + (r - nr)) + (g - ng)), H capped by the dirt height
__global__ void k2_thermal_out1(StepConsts c, const float* __restrict__ rock, const float* __restrict__ dirt,
                                float4* __restrict__ tc, float4* __restrict__ td) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y >= n) return;
    size_t i = at(n, x, y);
    const float r = rock[i], g = dirt[i];
    float dh[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        int xx = x + c2_ox[k], yy = y + c2_oy[k];
        bool in = inside(n, xx, yy);
        float nr = in ? rock[at(n, xx, yy)] : FAR_HEIGHT;
        float ng = in ? dirt[at(n, xx, yy)] : FAR_HEIGHT;
        dh[k] = (0.0f + (r - nr)) + (g - ng);
    }
    ThermalOut t = cell_thermal_dh(c.dt, c.Kalpha1, c.Kspeed1, g, dh);
    float o[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) o[k] = (t.mask >> k & 1u) ? t.S * dh[k] / t.bk : 0.0f;
    tc[i] = make_float4(o[0], o[1], o[2], o[3]);
    td[i] = make_float4(o[4], o[5], o[6], o[7]);
}

// glsl/smoothing.glsl:22-103, both channels
__global__ void k2_smooth(StepConsts c, const float* __restrict__ rock, const float* __restrict__ dirt,
                          float* __restrict__ rock_o, float* __restrict__ dirt_o) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y >= n) return;
    size_t i = at(n, x, y);
    float r = rock[i], g = dirt[i];
    if (!(x == 0 || y == 0 || x == n - 1 || y == n - 1))  // border texels are copied (:27-33)
        cell_smooth2(c.smooth_m, r, g, rock[i - 1], dirt[i - 1], rock[i + 1], dirt[i + 1], rock[i + n], dirt[i + n],
                     rock[i - n], dirt[i - n]);
    rock_o[i] = r;
    dirt_o[i] = g;
}

dim3 grid_for(int n) { return dim3((n + BX - 1) / BX, (n + BY - 1) / BY); }

}  // namespace

void launch_flux2(const StepConsts& c, const float* rock, const float* dirt, const float* water, const float* fl,
                  const float* fr, const float* ft, const float* fb, float* water_o, float* fl_o, float* fr_o,
                  float* ft_o, float* fb_o, float* u, float* v, float* vz, cudaStream_t st) {
    k2_flux<<<grid_for(c.n), dim3(BX, BY), 0, st>>>(c, rock, dirt, water, fl, fr, ft, fb, water_o, fl_o, fr_o, ft_o,
                                                     fb_o, u, v, vz);
    count_launch();
}

void launch_erosion2(const StepConsts& c, const float* u, const float* v, const float* vz, const float* rock,
                     const float* dirt, float* rock_o, float* dirt_o, float* s0, float* s1, cudaStream_t st) {
    k2_erosion<<<grid_for(c.n), dim3(BX, BY), 0, st>>>(c, u, v, vz, rock, dirt, rock_o, dirt_o, s0, s1);
    count_launch();
}

void launch_sediment2(const StepConsts& c, const float* u, const float* v, const float* s0, const float* s1,
                      float* s0_o, float* s1_o, float* water, cudaStream_t st) {
    k2_sediment<<<grid_for(c.n), dim3(BX, BY), 0, st>>>(c, u, v, s0, s1, s0_o, s1_o, water);
    count_launch();
}

void launch_thermal_out1(const StepConsts& c, const float* rock, const float* dirt, float4* tc, float4* td,
                         cudaStream_t st) {
    k2_thermal_out1<<<grid_for(c.n), dim3(BX, BY), 0, st>>>(c, rock, dirt, tc, td);
    count_launch();
}

void launch_smooth2(const StepConsts& c, const float* rock, const float* dirt, float* rock_o, float* dirt_o,
                    cudaStream_t st) {
    k2_smooth<<<grid_for(c.n), dim3(BX, BY), 0, st>>>(c, rock, dirt, rock_o, dirt_o);
    count_launch();
}

}  // namespace hg
