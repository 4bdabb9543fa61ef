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
