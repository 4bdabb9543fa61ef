// FP64 field totals for callers that cannot allocate device memory.
//
// hg_world_totals sums a world's fields with partial sums kept in scratch
// that hg_world_create allocated.  Some callers of this library cannot call
// cudaMalloc at all: a host application (a renderer or game engine, a
// content tool) that owns the device memory budget and hands plugins only
// the buffers it allocated, or a frame loop that cannot take the device-wide
// synchronisation cudaMalloc/cudaFree imply.  hg_field_totals_noalloc gives
// them the same reduction over buffers they already own: the partial sums
// live in the file-scope array below, sized for HG_NOALLOC_MAX_FIELDS
// fields, which every GPU that loads the library holds until the process
// exits.
#include "hg_internal.h"

namespace hg {

namespace {

constexpr int kParts = 304;  // blocks of the partial-sum kernel (2 per SM on 152 SMs)

// Partial sums: field f, block b at [f * kParts + b].  Each call writes every
// partial it later reads, so nothing here needs to start at zero.
static __device__ __align__(256) double g_noalloc_partials[HG_NOALLOC_MAX_FIELDS * kParts];

// The host-side name g_noalloc_partials is only a stand-in for the device
// array; kernels need its device address in the current context.  It is
// looked up on every call (a table lookup once the module is loaded, no
// allocation): a cached address would go stale when the context is
// destroyed and made again (cudaDeviceReset) and the module reloads
// elsewhere.
int partials_for_current_context(double** out, std::string& err) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        err = std::string("cudaGetSymbolAddress(g_noalloc_partials): ") + cudaGetErrorString(e);
        return HG_ERR_CUDA;
    }
    *out = static_cast<double*>(p);
    return HG_OK;
}

}  // namespace

}  // namespace hg

using namespace hg;

extern "C" int hg_field_totals_noalloc(const float* const* fields, int nfields, size_t count, double* out,
                                       void* stream) {
    if (!fields || !out) return hg_report_error(HG_ERR_INVALID, "hg_field_totals_noalloc: null fields or out");
    if (nfields < 1 || nfields > HG_NOALLOC_MAX_FIELDS)
        return hg_report_error(HG_ERR_INVALID,
                               "hg_field_totals_noalloc: nfields must be in [1, HG_NOALLOC_MAX_FIELDS = 8]");
    PtrList8 pl{};
    for (int f = 0; f < nfields; ++f) {
        if (!fields[f]) return hg_report_error(HG_ERR_INVALID, "hg_field_totals_noalloc: null field pointer");
        pl.p[f] = fields[f];
    }
    double* partials = nullptr;
    std::string err;
    int rc = partials_for_current_context(&partials, err);
    if (rc != HG_OK) return hg_report_error(rc, err.c_str());
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    launch_sum_f64(pl, nfields, count, partials, kParts, out, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return hg_report_error(HG_ERR_CUDA, (std::string("hg_field_totals_noalloc launch: ") +
                                             cudaGetErrorString(e)).c_str());
    return HG_OK;
}
