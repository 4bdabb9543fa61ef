// Device self-test of div_recip (hg_device.cuh) against IEEE division.
//
// No counterpart in the reference: it checks an arithmetic shortcut of this
// library.  Operands are drawn with Philox from the range div_recip's callers
// guarantee (a = 0 or |a| in [2^-80, 2^80], b in [2^-30, 2^40]); a third of
// them are built so that a/b lies next to a float (a = RN(q*b) nudged by up to
// two ulps) and a third next to the midpoint between two floats, the cases
// where a quotient rounds wrongly first.
#include "hg_internal.h"
#include "hg_tma.cuh"

namespace hg {
namespace {

__device__ __forceinline__ float uniform_exp_float(uint32_t w_exp, uint32_t w_man, int lo, int hi) {
    const int e = lo + (int)(w_exp % (uint32_t)(hi - lo + 1));
    return __uint_as_float((uint32_t)(e + 127) << 23 | (w_man & 0x7fffffu));
}

__global__ void k_selftest_division(uint32_t seed_lo, uint32_t seed_hi, unsigned long long count,
                                    unsigned long long* bad) {
    unsigned long long local = 0;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
        uint32_t w[4] = {(uint32_t)i, (uint32_t)(i >> 32), 0x5eedu, 0u};
        philox4x32_10(w, seed_lo, seed_hi);
        const float b = uniform_exp_float(w[0], w[1], -30, 39);
        float a;
        const uint32_t kind = w[3] % 3u;
        if (kind == 0) {
            a = uniform_exp_float(w[2], w[3] >> 2, -80, 79);
        } else {
            // a quotient q with |q*b| inside [2^-80, 2^80]
            const float q = uniform_exp_float(w[2], w[3] >> 2, -40, 39);
            if (kind == 1) {
                a = __fmul_rn(q, b);
                const int nudge = (int)((w[2] >> 24) % 5u) - 2;
                a = __int_as_float(__float_as_int(a) + nudge);
            } else {
                const double ulp = (double)__int_as_float(__float_as_int(q) + 1) - (double)q;
                a = (float)(((double)q + 0.5 * ulp) * (double)b);
            }
        }
        if ((w[1] >> 31) != 0) a = 0.0f;  // zero dividends
        if (!(a == 0.0f || (a >= 0x1p-80f && a <= 0x1p80f))) continue;
        const float y = __frcp_rn(b);
        if (__float_as_uint(div_recip(a, b, y)) != __float_as_uint(__fdiv_rn(a, b))) ++local;
        // the diagonal-slope form: divisor sqrt(2), dividend a drop in [2^-30, 2^40]
        const float dd = uniform_exp_float(w[2], w[0], -30, 39);
        if (__float_as_uint(div_recip(dd, SQRT2_F, RCP_SQRT2_F)) != __float_as_uint(__fdiv_rn(dd, SQRT2_F)))
            ++local;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && __float_as_uint(__frcp_rn(SQRT2_F)) != __float_as_uint(RCP_SQRT2_F))
        ++local;
    if (local) atomicAdd(bad, local);
}

// Paired f32x2 arithmetic against the scalar operations, lane by lane, on
// operands drawn from every float bit pattern (normal, subnormal, zero,
// infinite, NaN): counts in bad[0..4] the lanes where add2, mul2, fma2, sub2
// or div_recip2 differ from __fadd_rn, __fmul_rn, __fmaf_rn, __fsub_rn and
// div_recip, and in bad[5] where a product feeding a sum (gmix2, a Horner
// step) rounds other than twice (NaN results match any NaN).
__device__ __forceinline__ bool same_bits(float a, float b) {
    return __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b);
}
__global__ void k_selftest_paired(uint32_t seed_lo, uint32_t seed_hi, unsigned long long count,
                                  unsigned long long* bad) {
    unsigned long long local[6] = {0, 0, 0, 0, 0, 0};
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
        uint32_t w[4] = {(uint32_t)i, (uint32_t)(i >> 32), 0x9a17u, 0u};
        philox4x32_10(w, seed_lo, seed_hi);
        uint32_t v[4] = {(uint32_t)i, (uint32_t)(i >> 32), 0x9a18u, 0u};
        philox4x32_10(v, seed_lo, seed_hi);
        // one operand in eight subnormal (or zero), one in eight a signed zero
        float f[6];
        const uint32_t src[6] = {w[0], w[1], w[2], w[3], v[0], v[1]};
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            uint32_t bits = src[k];
            const uint32_t sel = (v[2] >> (3 * k)) & 7u;
            if (sel == 0) bits &= 0x807fffffu;
            else if (sel == 1) bits &= 0x80000000u;
            f[k] = __uint_as_float(bits);
        }
        const float2 a = make_float2(f[0], f[1]), b = make_float2(f[2], f[3]), c = make_float2(f[4], f[5]);
        const float2 s = add2(a, b), m = mul2(a, b), q = fma2(a, b, c), d = sub2(a, b);
        local[0] += !same_bits(s.x, __fadd_rn(a.x, b.x)) + !same_bits(s.y, __fadd_rn(a.y, b.y));
        local[1] += !same_bits(m.x, __fmul_rn(a.x, b.x)) + !same_bits(m.y, __fmul_rn(a.y, b.y));
        local[2] += !same_bits(q.x, __fmaf_rn(a.x, b.x, c.x)) + !same_bits(q.y, __fmaf_rn(a.y, b.y, c.y));
        local[3] += !same_bits(d.x, __fsub_rn(a.x, b.x)) + !same_bits(d.y, __fsub_rn(a.y, b.y));
        // div_recip2 on its callers' range
        const float bb0 = fabsf(b.x) >= 0x1p-30f && fabsf(b.x) <= 0x1p40f ? fabsf(b.x) : 1.5f;
        const float bb1 = fabsf(b.y) >= 0x1p-30f && fabsf(b.y) <= 0x1p40f ? fabsf(b.y) : 3.0f;
        const float aa0 = fabsf(a.x) >= 0x1p-80f && fabsf(a.x) <= 0x1p80f ? a.x : 0.0f;
        const float aa1 = fabsf(a.y) >= 0x1p-80f && fabsf(a.y) <= 0x1p80f ? a.y : 0.0f;
        const float2 y2 = make_float2(__frcp_rn(bb0), __frcp_rn(bb1));
        const float2 r = div_recip2(make_float2(aa0, aa1), make_float2(-bb0, -bb1), y2);
        local[4] += !same_bits(r.x, div_recip(aa0, bb0, y2.x)) + !same_bits(r.y, div_recip(aa1, bb1, y2.y));
        // products feeding sums: a mix with a weight in [0, 1), a Horner step
        const float2 wt = make_float2((w[0] >> 8) * 0x1p-24f, (w[1] >> 8) * 0x1p-24f);
        const float2 g = gmix2(a, b, wt), hs = add2(mul2(a, b), c);
        local[5] += !same_bits(g.x, gmix(a.x, b.x, wt.x)) + !same_bits(g.y, gmix(a.y, b.y, wt.y));
        local[5] += !same_bits(hs.x, __fadd_rn(__fmul_rn(a.x, b.x), c.x)) +
                    !same_bits(hs.y, __fadd_rn(__fmul_rn(a.y, b.y), c.y));
    }
#pragma unroll
    for (int k = 0; k < 6; ++k)
        if (local[k]) atomicAdd(bad + k, local[k]);
}

// The kernels' bounded wait on a barrier phase that never completes: one
// arrival is expected and none comes, and no copy is in flight.  Thread 0
// records whether the wait gave up and how long `polls` polls took.
__global__ void k_selftest_wait(uint32_t polls, int* timed_out, unsigned long long* ns) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    unsigned long long t0, t1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    const bool ok = __syncthreads_and(mbar_wait_n(&bar, 0, polls));
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
    if (threadIdx.x == 0) {
        *timed_out = ok ? 0 : 1;
        *ns = t1 - t0;
    }
}

}  // namespace
}  // namespace hg

extern "C" int hg_selftest_bounded_wait(uint32_t polls, int* timed_out, double* ns_per_poll) {
    using namespace hg;
    if (!timed_out || !ns_per_poll) return hg_report_error(HG_ERR_INVALID, "null output pointer");
    if (polls < 1 || polls > kMaxPolls) return hg_report_error(HG_ERR_INVALID, "polls must be in [1, 2^18]");
    int* d = nullptr;
    cudaError_t e = cudaMalloc((void**)&d, 16);
    if (e == cudaSuccess) e = cudaMemset(d, 0, 16);
    if (e == cudaSuccess) {
        k_selftest_wait<<<1, 32>>>(polls, d, reinterpret_cast<unsigned long long*>(d + 2));
        count_launch();
        e = cudaGetLastError();
    }
    int flag = 0;
    unsigned long long ns = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&flag, d, sizeof(flag), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&ns, d + 2, sizeof(ns), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return hg_report_error(HG_ERR_CUDA, cudaGetErrorString(e));
    *timed_out = flag;
    *ns_per_poll = (double)ns / polls;
    return HG_OK;
}

extern "C" int hg_selftest_division(uint64_t seed, uint64_t count, uint64_t* mismatches) {
    using namespace hg;
    if (!mismatches) return hg_report_error(HG_ERR_INVALID, "null output pointer");
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMalloc((void**)&d, sizeof(*d));
    if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(*d));
    if (e == cudaSuccess) {
        k_selftest_division<<<4 * 152, 256>>>((uint32_t)seed, (uint32_t)(seed >> 32), count, d);
        count_launch();
        e = cudaGetLastError();
    }
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return hg_report_error(HG_ERR_CUDA, cudaGetErrorString(e));
    *mismatches = h;
    return HG_OK;
}

extern "C" int hg_selftest_paired(uint64_t seed, uint64_t count, uint64_t mismatches[6]) {
    using namespace hg;
    if (!mismatches) return hg_report_error(HG_ERR_INVALID, "null output pointer");
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMalloc((void**)&d, 6 * sizeof(*d));
    if (e == cudaSuccess) e = cudaMemset(d, 0, 6 * sizeof(*d));
    if (e == cudaSuccess) {
        k_selftest_paired<<<4 * 152, 256>>>((uint32_t)seed, (uint32_t)(seed >> 32), count, d);
        count_launch();
        e = cudaGetLastError();
    }
    unsigned long long h[6] = {0, 0, 0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return hg_report_error(HG_ERR_CUDA, cudaGetErrorString(e));
    for (int k = 0; k < 6; ++k) mismatches[k] = h[k];
    return HG_OK;
}
