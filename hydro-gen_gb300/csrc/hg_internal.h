// Internal declarations shared by the library's translation units.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/hydrogen.h"
#include "hg_device.cuh"

namespace hg {

// Carried state fields, in the order of the HG_FIELD_* ids 0..6.
enum { S_ROCK = 0, S_WATER, S_SED, S_FL, S_FR, S_FT, S_FB, S_COUNT };

struct StateBufs {
    float* f[S_COUNT];
};

extern std::atomic<uint64_t> g_launches;
inline void count_launch(uint64_t k = 1) { g_launches.fetch_add(k, std::memory_order_relaxed); }

// ---- per-pass kernels (hg_plain.cu) --------------------------------------------
void launch_rain(const StepConsts& c, const RainStep& r, float* water, cudaStream_t st);
void launch_flux(const StepConsts& c, const float* rock, const float* water, const float* fl, const float* fr,
                 const float* ft, const float* fb, float* water_o, float* fl_o, float* fr_o, float* ft_o,
                 float* fb_o, float* u, float* v, float* vz, cudaStream_t st);
void launch_erosion(const StepConsts& c, const float* u, const float* v, const float* vz, const float* rock,
                    float* rock_o, float* sed_inout, cudaStream_t st);
void launch_sediment(const StepConsts& c, const float* u, const float* v, const float* sed, float* sed_o,
                     float* water_inout, cudaStream_t st);
void launch_thermal_out(const StepConsts& c, const float* rock, float4* tc, float4* td, cudaStream_t st);
void launch_thermal_in(const StepConsts& c, const float* rock, const float4* tc, const float4* td,
                       float* rock_o, cudaStream_t st);

// ---- fused step (hg_fused.cu) ---------------------------------------------------
struct FusedArgs {
    StepConsts c;
    RainStep rain[8];  // per sub-step
    StateBufs in, out;
    float* u;
    float* v;
    float* s_ero;  // eroded sediment of every cell (k_hydro -> k_transport)
    float* b_ero;  // eroded rock of every cell (k_hydro -> k_transport, thermal on)
    int* err;      // set to 1 when a bounded wait for a TMA tile gives up
};

// TMA tensor maps of the fused step: rock, water, sediment, fL, fR, fT, fB
// (k_hydro boxes) and eroded rock (k_transport box).
struct TmaMaps {
    CUtensorMap m[8];
};
// Tensor maps encoded once per (buffer, box) and reused.
struct TmaCache {
    struct Entry {
        const float* base;
        int n, box_h;
        CUtensorMap map;
    };
    std::vector<Entry> entries;
    bool get(const float* base, int n, int box_h, CUtensorMap* out);
};

int fused_max_depth();
// Launches k_hydro and k_transport for one step; false if a tensor map could
// not be encoded.
bool launch_fused(const FusedArgs& a, TmaCache& cache, cudaStream_t st);
// The fused kernel's tile shape and depth currently compiled in.
bool fused_supported(int depth, int tile_x, int tile_y);

// ---- init and reductions (hg_init.cu) ---------------------------------------------
void launch_fbm_raw(float* out, int n, const hg_noise_settings& s, cudaStream_t st);
// min and max of a device array into two floats of `minmax` (device).
void launch_minmax(const float* x, size_t count, float* partial, int nparts, float* minmax, cudaStream_t st);
void launch_scale(float* x, size_t count, const float* minmax, float lo, float hi, cudaStream_t st);
void launch_ks_from_fbm(float* x, size_t count, float base, float k_over_amp, cudaStream_t st);
// Deterministic FP64 sum of up to 8 arrays: out[i] = sum of field i.
struct PtrList8 { const float* p[8]; };
void launch_sum_f64(const PtrList8& fields, int nfields, size_t count, double* partial, int nparts,
                    double* out, cudaStream_t st);
int reduction_parts();

// host copy of the polynomial arctangent (same operations as poly_atanf)
float host_poly_atanf(float x);

// Records msg as this thread's hg_last_error() and returns code.
int hg_report_error(int code, const char* msg);

}  // namespace hg
