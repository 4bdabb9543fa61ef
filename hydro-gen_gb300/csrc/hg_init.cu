// Heightmap initialisation (simplex fBm) and grid reductions.
//
// The heightmap generator replaces World::gen_heightmap's dispatch of
// glsl/heightmap.glsl (src/state.cpp:116-147) with the workload's simplex fBm:
// a 2-D simplex noise written from Gustavson's description ("Simplex noise
// demystified", 2005) with an integer corner hash (MurmurHash3's finaliser),
// summed over octaves and min-max scaled.  Every float operation is written
// out in a fixed order so the float CPU restatement reproduces it bit for bit.
#include "hg_internal.h"

namespace hg {

namespace {

__device__ __forceinline__ uint32_t fmix32(uint32_t h) {
    h ^= h >> 16; h *= 0x85ebca6bu; h ^= h >> 13; h *= 0xc2b2ae35u; h ^= h >> 16;
    return h;
}
__device__ __forceinline__ uint32_t corner_hash(int32_t i, int32_t j, uint32_t seed) {
    return fmix32((uint32_t)i * 0x8da6b343u ^ (uint32_t)j * 0xd8163841u ^ seed * 0xcb1ab31fu);
}
__device__ __forceinline__ float grad_dot(uint32_t h, float x, float y) {
    switch (h & 7u) {  // (+-1,+-1), (+-1,0), (0,+-1)
        case 0: return x + y;
        case 1: return -x + y;
        case 2: return x - y;
        case 3: return -x - y;
        case 4: return x;
        case 5: return -x;
        case 6: return y;
        default: return -y;
    }
}

__device__ float simplex2f(float x, float y, uint32_t seed) {
    const float F2 = 0.366025403784f;  // (sqrt(3)-1)/2: skew to the simplex lattice
    const float G2 = 0.211324865405f;  // (3-sqrt(3))/6: unskew
    float s = (x + y) * F2;
    float fi = floorf(x + s), fj = floorf(y + s);
    float t = (fi + fj) * G2;
    float x0 = x - (fi - t), y0 = y - (fj - t);
    int i1 = x0 > y0 ? 1 : 0, j1 = 1 - i1;
    float x1 = x0 - (float)i1 + G2, y1 = y0 - (float)j1 + G2;
    float x2 = x0 - 1.0f + 2.0f * G2, y2 = y0 - 1.0f + 2.0f * G2;
    int32_t i = (int32_t)fi, j = (int32_t)fj;
    float nsum = 0.0f;
    float t0 = 0.5f - x0 * x0 - y0 * y0;
    if (t0 > 0.0f) { t0 = t0 * t0; nsum = nsum + t0 * t0 * grad_dot(corner_hash(i, j, seed), x0, y0); }
    float t1 = 0.5f - x1 * x1 - y1 * y1;
    if (t1 > 0.0f) { t1 = t1 * t1; nsum = nsum + t1 * t1 * grad_dot(corner_hash(i + i1, j + j1, seed), x1, y1); }
    float t2 = 0.5f - x2 * x2 - y2 * y2;
    if (t2 > 0.0f) { t2 = t2 * t2; nsum = nsum + t2 * t2 * grad_dot(corner_hash(i + 1, j + 1, seed), x2, y2); }
    return 70.0f * nsum;
}

__global__ void k_fbm(float* __restrict__ out, int n, hg_noise_settings s) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= n || y >= n) return;
    float sum = 0.0f, amp = 1.0f, f = s.frequency;
    for (int o = 0; o < s.octaves; ++o) {
        sum = sum + amp * simplex2f((float)x * f, (float)y * f, s.seed + (uint32_t)o);
        amp = amp * s.gain;
        f = f * s.lacunarity;
    }
    out[(size_t)y * n + x] = sum;
}

constexpr int RED_THREADS = 512;
constexpr int RED_PARTS = 304;  // 2 blocks per SM on 152 SMs

__global__ void k_minmax_part(const float* __restrict__ x, size_t count, float* __restrict__ part) {
    float mn = INFINITY, mx = -INFINITY;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        float v = x[i];
        mn = fminf(mn, v);
        mx = fmaxf(mx, v);
    }
    __shared__ float smn[RED_THREADS / 32], smx[RED_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { smn[wid] = mn; smx[wid] = mx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) { mn = fminf(mn, smn[k]); mx = fmaxf(mx, smx[k]); }
        part[2 * blockIdx.x] = mn;
        part[2 * blockIdx.x + 1] = mx;
    }
}

__global__ void k_minmax_final(const float* __restrict__ part, int nparts, float* __restrict__ mm) {
    if (threadIdx.x != 0) return;
    float mn = part[0], mx = part[1];
    for (int k = 1; k < nparts; ++k) { mn = fminf(mn, part[2 * k]); mx = fmaxf(mx, part[2 * k + 1]); }
    mm[0] = mn; mm[1] = mx;
}

// lo + ((v - min) / (max - min)) * (hi - lo)
__global__ void k_scale(float* __restrict__ x, size_t count, const float* __restrict__ mm, float lo, float hi) {
    float mn = mm[0], range = mm[1] - mm[0], span = hi - lo;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        x[i] = lo + ((x[i] - mn) / range) * span;
}

__global__ void k_ks(float* __restrict__ x, size_t count, float base, float k_over_amp) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        x[i] = base * expf(k_over_amp * x[i]);
}

// Deterministic FP64 sums: fixed grid, fixed per-thread stride, fixed tree.
__global__ void k_sum_part(PtrList8 fields, int nfields, size_t count, double* __restrict__ part) {
    __shared__ double sh[RED_THREADS / 32];
    for (int f = 0; f < nfields; ++f) {
        const float* x = fields.p[f];
        double acc = 0.0;
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
            acc += (double)x[i];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
        if (lane == 0) sh[wid] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
            part[(size_t)f * gridDim.x + blockIdx.x] = t;
        }
        __syncthreads();
    }
}

__global__ void k_sum_final(const double* __restrict__ part, int nparts, int nfields, double* __restrict__ out) {
    int f = threadIdx.x;
    if (f >= nfields) return;
    double t = 0.0;
    for (int k = 0; k < nparts; ++k) t += part[(size_t)f * nparts + k];
    out[f] = t;
}

}  // namespace

int reduction_parts() { return RED_PARTS; }

void launch_fbm_raw(float* out, int n, const hg_noise_settings& s, cudaStream_t st) {
    dim3 blk(32, 8), grd((n + 31) / 32, (n + 7) / 8);
    k_fbm<<<grd, blk, 0, st>>>(out, n, s);
    count_launch();
}

void launch_minmax(const float* x, size_t count, float* partial, int nparts, float* minmax, cudaStream_t st) {
    k_minmax_part<<<nparts, RED_THREADS, 0, st>>>(x, count, partial);
    k_minmax_final<<<1, 32, 0, st>>>(partial, nparts, minmax);
    count_launch(2);
}

void launch_scale(float* x, size_t count, const float* minmax, float lo, float hi, cudaStream_t st) {
    k_scale<<<RED_PARTS * 4, 256, 0, st>>>(x, count, minmax, lo, hi);
    count_launch();
}

void launch_ks_from_fbm(float* x, size_t count, float base, float k_over_amp, cudaStream_t st) {
    k_ks<<<RED_PARTS * 4, 256, 0, st>>>(x, count, base, k_over_amp);
    count_launch();
}

// NaN and infinite values of x (exponent bits all ones), added to *out
__global__ void k_nonfinite(const float* __restrict__ x, size_t count, unsigned long long* __restrict__ out) {
    unsigned long long k = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        k += (__float_as_uint(x[i]) & 0x7f800000u) == 0x7f800000u ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
    if ((threadIdx.x & 31) == 0 && k) atomicAdd(out, k);
}

void launch_count_nonfinite(const float* x, size_t count, unsigned long long* out, cudaStream_t st) {
    k_nonfinite<<<RED_PARTS * 4, 256, 0, st>>>(x, count, out);
    count_launch();
}

void launch_sum_f64(const PtrList8& fields, int nfields, size_t count, double* partial, int nparts,
                    double* out, cudaStream_t st) {
    k_sum_part<<<nparts, RED_THREADS, 0, st>>>(fields, nfields, count, partial);
    k_sum_final<<<1, 32, 0, st>>>(partial, nparts, nfields, out);
    count_launch(2);
}

}  // namespace hg
