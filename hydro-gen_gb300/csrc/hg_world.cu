// Host side of the C ABI: worlds, settings, step sequencing, transfers.
//
// A world owns its device fields (FP32 structure-of-arrays, n*n floats each,
// double-buffered where a pass reads neighbours), one CUDA stream and a few
// reduction scratch buffers.  hg_step sequences the passes the way
// Erosion::dispatch_grid does (src/erosion.cpp:158-200), swapping buffer
// pointers where the reference swaps Tex_pair read/write textures.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "hg_internal.h"

namespace hg {
std::atomic<uint64_t> g_launches{0};

// Same operations as poly_atanf in hg_device.cuh; volatile keeps one
// rounding per operation whatever the host compiler's contraction rules.
static float host_poly_atan_core(float u) {
    const float c0 = -3.333333135e-01f, c1 = 1.999990344e-01f, c2 = -1.428200752e-01f,
                c3 = 1.104469076e-01f, c4 = -8.476266265e-02f, c5 = 4.744043201e-02f;
    volatile float s = u * u;
    volatile float p = c5;
    p = p * s; p = p + c4;
    p = p * s; p = p + c3;
    p = p * s; p = p + c2;
    p = p * s; p = p + c1;
    p = p * s; p = p + c0;
    volatile float q = s * p;
    q = u * q;
    volatile float r = u + q;
    return r;
}

float host_poly_atanf(float x) {
    volatile float ax = std::fabs(x);
    volatile float r;
    if (ax <= 0.414213562f) {
        r = host_poly_atan_core(ax);
    } else if (ax <= 2.41421356f) {
        volatile float nu = ax - 1.0f, de = ax + 1.0f;
        volatile float u = nu / de;
        r = 0.785398163f + host_poly_atan_core(u);
    } else {
        volatile float u = 1.0f / ax;
        r = 1.57079637f - host_poly_atan_core(u);
    }
    return std::copysign((float)r, x);
}
}  // namespace hg

using namespace hg;

struct hg_world {
    int n = 0;
    int layers = 1;
    int device = 0;
    cudaStream_t stream = nullptr;
    hg_erosion_settings es{};
    hg_rain_settings rs{};
    hg_step_options opt{};
    uint64_t step = 0;
    float* cur[S_COUNT] = {};
    float* alt[S_COUNT] = {};
    float* u = nullptr;
    float* v = nullptr;
    float* vz = nullptr;
    float4* tc = nullptr;
    float4* td = nullptr;
    float* ks = nullptr;
    bool ks_on = false;
    float* s_ero = nullptr;  // fused step: eroded sediment of every cell
    float* b_ero = nullptr;  // fused step: eroded rock of every cell
    int* err = nullptr;      // device flag: a bounded wait gave up
    TmaCache tma;
    float* red_f = nullptr;   // min/max partials + result
    double* red_d = nullptr;  // FP64 partials + result
};

namespace {

thread_local std::string t_err;

int fail(int code, const std::string& msg) {
    t_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    cudaGetLastError();  // clear a sticky launch error so later calls report their own
    return fail(HG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define HG_CUDA(call)                                   \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

#define HG_CHECK_WORLD(w) \
    if (!(w)) return fail(HG_ERR_INVALID, "null world")

// Make the world's device current for the duration of a call.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int now = -1;
        if (prev >= 0 && cudaGetDevice(&now) == cudaSuccess && now != prev) cudaSetDevice(prev);
    }
};

size_t cells(const hg_world* w) { return (size_t)w->n * w->n; }

void free_world(hg_world* w) {
    for (int f = 0; f < S_COUNT; ++f) {
        cudaFree(w->cur[f]);
        cudaFree(w->alt[f]);
    }
    cudaFree(w->u); cudaFree(w->v); cudaFree(w->vz);
    cudaFree(w->tc); cudaFree(w->td);
    cudaFree(w->ks);
    cudaFree(w->s_ero); cudaFree(w->b_ero); cudaFree(w->err);
    cudaFree(w->red_f); cudaFree(w->red_d);
    if (w->stream) cudaStreamDestroy(w->stream);
}

// Smallest float x >= 0 with host_poly_atanf(x) > alpha (the arctangent is
// monotone on x >= 0, so this splits the axis); NaN when no float qualifies.
float talus_cross_threshold(float alpha) {
    auto pred = [&](uint32_t bits) {
        float x;
        std::memcpy(&x, &bits, 4);
        return host_poly_atanf(x) > alpha;
    };
    uint32_t lo = 0, hi = 0x7f800000u;  // +0 .. +inf
    if (!pred(hi)) return NAN;
    if (pred(lo)) return 0.0f;
    while (hi - lo > 1) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (pred(mid)) hi = mid; else lo = mid;
    }
    float x;
    std::memcpy(&x, &hi, 4);
    return x;
}

// Smallest float drop b >= 0 with b / sqrt(2) (rounded) >= xc; NaN if none.
float talus_diag_threshold(float xc) {
    if (std::isnan(xc)) return NAN;
    auto pred = [&](uint32_t bits) {
        float b;
        std::memcpy(&b, &bits, 4);
        volatile float q = b / 1.41421354f;
        return q >= xc;
    };
    uint32_t lo = 0, hi = 0x7f800000u;
    if (!pred(hi)) return NAN;
    if (pred(lo)) return 0.0f;
    while (hi - lo > 1) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (pred(mid)) hi = mid; else lo = mid;
    }
    float b;
    std::memcpy(&b, &hi, 4);
    return b;
}

bool thermal_on(const hg_world* w) {
    if (w->opt.thermal == HG_AUTO) return w->es.Kspeed[0] != 0.0f;
    return w->opt.thermal != 0;
}

StepConsts make_consts(const hg_world* w) {
    StepConsts c{};
    const hg_erosion_settings& s = w->es;
    volatile float dt = s.d_t;  // products rounded once, as the shaders do per cell
    c.n = w->n;
    c.dt = s.d_t;
    c.G = s.G;
    c.EK = s.ENERGY_KEPT;
    c.Kc = s.Kc;
    c.Kls0 = dt * s.Ks[0];
    c.Kld0 = dt * s.Kd[0];
    c.Kls1 = dt * s.Ks[1];
    c.Kld1 = dt * s.Kd[1];
    c.Ks0 = s.Ks[0];
    c.ks_field = w->ks_on ? w->ks : nullptr;
    volatile float ke_dt = s.Ke * dt;
    c.evap = 1.0f - ke_dt;
    c.Kalpha0 = s.Kalpha[0];
    c.Kspeed0 = s.Kspeed[0];
    c.thermal = thermal_on(w) ? 1 : 0;
    c.talus_x_cross = talus_cross_threshold(s.Kalpha[0]);
    c.talus_b_diag = talus_diag_threshold(c.talus_x_cross);
    return c;
}

RainStep make_rain(const hg_world* w, uint64_t step1) {
    RainStep r{};
    const hg_step_options& o = w->opt;
    int period = w->rs.period;
    r.active = (o.rain_mode != HG_RAIN_OFF && period > 0 && step1 % (uint64_t)period == 0) ? 1 : 0;
    r.bernoulli = o.rain_mode == HG_RAIN_BERNOULLI ? 1 : 0;
    r.amount = w->rs.amount;
    double t = std::floor((double)o.rain_probability * 4294967296.0);
    if (t < 0) t = 0;
    if (t > 4294967295.0) t = 4294967295.0;
    r.threshold = (uint32_t)t;
    r.seed_lo = (uint32_t)o.rain_seed;
    r.seed_hi = (uint32_t)(o.rain_seed >> 32);
    r.terrain_id = o.terrain_id;
    r.step = (uint32_t)step1;
    return r;
}

bool pick_tile(const hg_world* w, int& tx, int& ty) {
    const int cand[][2] = {{64, 16}};
    if (w->opt.tile_x > 0 && w->opt.tile_y > 0) {
        tx = w->opt.tile_x; ty = w->opt.tile_y;
        return fused_supported(1, tx, ty) && w->n % tx == 0 && w->n % ty == 0;
    }
    for (auto& cxy : cand)
        if (w->n % cxy[0] == 0 && w->n % cxy[1] == 0) { tx = cxy[0]; ty = cxy[1]; return true; }
    return false;
}

float* field_ptr(hg_world* w, int field) {
    switch (field) {
        case HG_FIELD_ROCK: return w->cur[S_ROCK];
        case HG_FIELD_WATER: return w->cur[S_WATER];
        case HG_FIELD_SEDIMENT: return w->cur[S_SED];
        case HG_FIELD_FLUX_L: return w->cur[S_FL];
        case HG_FIELD_FLUX_R: return w->cur[S_FR];
        case HG_FIELD_FLUX_T: return w->cur[S_FT];
        case HG_FIELD_FLUX_B: return w->cur[S_FB];
        case HG_FIELD_VEL_U: return w->u;
        case HG_FIELD_VEL_V: return w->v;
        case HG_FIELD_VEL_Z: return w->vz;
        case HG_FIELD_KS: return w->ks;
    }
    return nullptr;
}

}  // namespace

int hg::hg_report_error(int code, const char* msg) { return fail(code, msg); }

extern "C" {

const char* hg_version(void) { return "hydrogen-gb300 0.1 (sm_103a)"; }
const char* hg_last_error(void) { return t_err.c_str(); }
uint64_t hg_launch_count(void) { return g_launches.load(); }

int hg_default_erosion_settings(hg_erosion_settings* out) {
    if (!out) return fail(HG_ERR_INVALID, "null settings");
    std::memset(out, 0, sizeof(*out));
    // grid-model defaults, src/state.cpp:81-92
    out->Kc = 0.2f;
    out->Kalpha[0] = 1.3f; out->Kalpha[1] = 0.6f;
    out->Kconv = 0.001f;
    out->Ks[0] = 0.03f; out->Ks[1] = 0.09f;
    out->Kd[0] = 0.01f; out->Kd[1] = 0.03f;
    out->Ke = 0.03f;
    out->ENERGY_KEPT = 1.0f;
    out->Kspeed[0] = 0.5f; out->Kspeed[1] = 2.0f;
    out->G = 1.0f;
    out->d_t = 0.001f;
    return HG_OK;
}

int hg_default_rain_settings(hg_rain_settings* out) {
    if (!out) return fail(HG_ERR_INVALID, "null settings");
    // src/settings.hpp:16-21
    out->amount = 0.01f;
    out->mountain_thresh = 0.55f;
    out->mountain_multip = 0.05f;
    out->period = 512;
    out->drops = 0.02f;
    return HG_OK;
}

int hg_default_step_options(hg_step_options* out) {
    if (!out) return fail(HG_ERR_INVALID, "null options");
    std::memset(out, 0, sizeof(*out));
    out->rain_mode = HG_RAIN_OFF;
    out->thermal = HG_AUTO;
    out->temporal_depth = HG_AUTO;
    out->tile_x = HG_AUTO;
    out->tile_y = HG_AUTO;
    return HG_OK;
}

int hg_world_create(int n, int layers, hg_world** out) {
    if (!out) return fail(HG_ERR_INVALID, "null output pointer");
    *out = nullptr;
    if (n <= 0 || n % 8 != 0) return fail(HG_ERR_INVALID, "n must be a positive multiple of 8");
    if (layers != 1) return fail(HG_ERR_UNSUPPORTED, "only the one-layer (rock) world is supported");
    hg_world* w = new (std::nothrow) hg_world();
    if (!w) return fail(HG_ERR_OOM, "host allocation failed");
    w->n = n;
    w->layers = layers;
    cudaGetDevice(&w->device);
    hg_default_erosion_settings(&w->es);
    w->es.Kconv = 0.0f;       // one-layer world: no dirt layer to convert into
    w->es.Kspeed[1] = 0.0f;
    hg_default_rain_settings(&w->rs);
    hg_default_step_options(&w->opt);
    size_t bytes = (size_t)n * n * sizeof(float);
    auto alloc = [&](void** p, size_t b) -> cudaError_t { return cudaMalloc(p, b); };
    cudaError_t e = cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking);
    for (int f = 0; f < S_COUNT && e == cudaSuccess; ++f) {
        e = alloc((void**)&w->cur[f], bytes);
        if (e == cudaSuccess) e = alloc((void**)&w->alt[f], bytes);
    }
    if (e == cudaSuccess) e = alloc((void**)&w->u, bytes);
    if (e == cudaSuccess) e = alloc((void**)&w->v, bytes);
    if (e == cudaSuccess) e = alloc((void**)&w->vz, bytes);
    if (e == cudaSuccess) e = alloc((void**)&w->tc, 4 * bytes);
    if (e == cudaSuccess) e = alloc((void**)&w->td, 4 * bytes);
    if (e == cudaSuccess) e = alloc((void**)&w->ks, bytes);
    if (e == cudaSuccess) e = alloc((void**)&w->s_ero, bytes);
    if (e == cudaSuccess) e = alloc((void**)&w->b_ero, bytes);
    if (e == cudaSuccess) e = alloc((void**)&w->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(w->err, 0, sizeof(int), w->stream);
    if (e == cudaSuccess) e = alloc((void**)&w->red_f, sizeof(float) * (2 * reduction_parts() + 2));
    if (e == cudaSuccess) e = alloc((void**)&w->red_d, sizeof(double) * (8 * reduction_parts() + 8));
    if (e != cudaSuccess) {
        free_world(w);
        delete w;
        int code = e == cudaErrorMemoryAllocation ? HG_ERR_OOM : HG_ERR_CUDA;
        cudaGetLastError();
        return fail(code, std::string("world allocation: ") + cudaGetErrorString(e));
    }
    for (int f = 0; f < S_COUNT; ++f) {
        cudaMemsetAsync(w->cur[f], 0, bytes, w->stream);
        cudaMemsetAsync(w->alt[f], 0, bytes, w->stream);
    }
    cudaMemsetAsync(w->u, 0, bytes, w->stream);
    cudaMemsetAsync(w->v, 0, bytes, w->stream);
    cudaMemsetAsync(w->vz, 0, bytes, w->stream);
    e = cudaStreamSynchronize(w->stream);
    if (e != cudaSuccess) {
        free_world(w);
        delete w;
        return cuda_fail(e, "world zero-fill");
    }
    *out = w;
    return HG_OK;
}

int hg_world_destroy(hg_world* w) {
    if (!w) return HG_OK;
    DeviceGuard g(w->device);
    cudaStreamSynchronize(w->stream);
    free_world(w);
    delete w;
    return HG_OK;
}

int hg_world_size(const hg_world* w, int* n) {
    HG_CHECK_WORLD(w);
    if (!n) return fail(HG_ERR_INVALID, "null output");
    *n = w->n;
    return HG_OK;
}

int hg_world_stream(const hg_world* w, void** stream) {
    HG_CHECK_WORLD(w);
    if (!stream) return fail(HG_ERR_INVALID, "null output");
    *stream = (void*)w->stream;
    return HG_OK;
}

int hg_set_erosion_settings(hg_world* w, const hg_erosion_settings* s) {
    HG_CHECK_WORLD(w);
    if (!s) return fail(HG_ERR_INVALID, "null settings");
    if (s->particle_count != 0) return fail(HG_ERR_INVALID, "particle_count must be 0 for the grid model");
    if (!(s->d_t > 0.0f) || !std::isfinite(s->d_t)) return fail(HG_ERR_INVALID, "d_t must be positive and finite");
    if (w->layers == 1 && s->Kconv != 0.0f)
        return fail(HG_ERR_INVALID, "Kconv must be 0 in a one-layer world (no dirt layer)");
    if (w->layers == 1 && s->Kspeed[1] != 0.0f)
        return fail(HG_ERR_INVALID, "Kspeed[1] must be 0 in a one-layer world (dirt slippage and smoothing)");
    w->es = *s;
    return HG_OK;
}

int hg_get_erosion_settings(const hg_world* w, hg_erosion_settings* s) {
    HG_CHECK_WORLD(w);
    if (!s) return fail(HG_ERR_INVALID, "null settings");
    *s = w->es;
    return HG_OK;
}

int hg_set_rain_settings(hg_world* w, const hg_rain_settings* s) {
    HG_CHECK_WORLD(w);
    if (!s) return fail(HG_ERR_INVALID, "null settings");
    if (s->period < 0) return fail(HG_ERR_INVALID, "rain period must be >= 0");
    w->rs = *s;
    return HG_OK;
}

int hg_set_step_options(hg_world* w, const hg_step_options* o) {
    HG_CHECK_WORLD(w);
    if (!o) return fail(HG_ERR_INVALID, "null options");
    if (o->rain_mode < HG_RAIN_OFF || o->rain_mode > HG_RAIN_BERNOULLI) return fail(HG_ERR_INVALID, "bad rain_mode");
    if (!(o->rain_probability >= 0.0f && o->rain_probability <= 1.0f))
        return fail(HG_ERR_INVALID, "rain_probability must be in [0, 1]");
    if (o->temporal_depth != HG_AUTO && (o->temporal_depth < 1 || o->temporal_depth > fused_max_depth()))
        return fail(HG_ERR_UNSUPPORTED, "temporal_depth out of the supported range");
    w->opt = *o;
    return HG_OK;
}

int hg_init_heightmap(hg_world* w, const hg_noise_settings* s) {
    HG_CHECK_WORLD(w);
    if (!s) return fail(HG_ERR_INVALID, "null noise settings");
    if (s->octaves < 1 || s->octaves > 32) return fail(HG_ERR_INVALID, "octaves must be in [1, 32]");
    DeviceGuard g(w->device);
    size_t bytes = cells(w) * sizeof(float);
    for (int f = 0; f < S_COUNT; ++f) {
        HG_CUDA(cudaMemsetAsync(w->cur[f], 0, bytes, w->stream));
        HG_CUDA(cudaMemsetAsync(w->alt[f], 0, bytes, w->stream));
    }
    HG_CUDA(cudaMemsetAsync(w->u, 0, bytes, w->stream));
    HG_CUDA(cudaMemsetAsync(w->v, 0, bytes, w->stream));
    HG_CUDA(cudaMemsetAsync(w->vz, 0, bytes, w->stream));
    launch_fbm_raw(w->cur[S_ROCK], w->n, *s, w->stream);
    launch_minmax(w->cur[S_ROCK], cells(w), w->red_f, reduction_parts(), w->red_f + 2 * reduction_parts(),
                  w->stream);
    launch_scale(w->cur[S_ROCK], cells(w), w->red_f + 2 * reduction_parts(), s->out_min, s->out_max, w->stream);
    HG_CUDA(cudaGetLastError());
    w->step = 0;
    return HG_OK;
}

int hg_init_ks_field(hg_world* w, const hg_noise_settings* s, float base, float k) {
    HG_CHECK_WORLD(w);
    if (!s) return fail(HG_ERR_INVALID, "null noise settings");
    if (s->octaves < 1 || s->octaves > 32) return fail(HG_ERR_INVALID, "octaves must be in [1, 32]");
    DeviceGuard g(w->device);
    float amp = 0.0f, a = 1.0f;
    for (int o = 0; o < s->octaves; ++o) { amp += a; a *= s->gain; }
    launch_fbm_raw(w->ks, w->n, *s, w->stream);
    launch_ks_from_fbm(w->ks, cells(w), base, k / amp, w->stream);
    HG_CUDA(cudaGetLastError());
    w->ks_on = true;
    return HG_OK;
}

int hg_clear_ks_field(hg_world* w) {
    HG_CHECK_WORLD(w);
    w->ks_on = false;
    return HG_OK;
}

int hg_world_upload(hg_world* w, int field, const float* host) {
    HG_CHECK_WORLD(w);
    if (!host) return fail(HG_ERR_INVALID, "null host pointer");
    float* d = field_ptr(w, field);
    if (!d) return fail(HG_ERR_INVALID, "bad field id");
    DeviceGuard g(w->device);
    HG_CUDA(cudaMemcpyAsync(d, host, cells(w) * sizeof(float), cudaMemcpyHostToDevice, w->stream));
    HG_CUDA(cudaStreamSynchronize(w->stream));
    if (field == HG_FIELD_KS) w->ks_on = true;
    return HG_OK;
}

int hg_world_download(hg_world* w, int field, float* host) {
    HG_CHECK_WORLD(w);
    if (!host) return fail(HG_ERR_INVALID, "null host pointer");
    float* d = field_ptr(w, field);
    if (!d) return fail(HG_ERR_INVALID, "bad field id");
    DeviceGuard g(w->device);
    HG_CUDA(cudaMemcpyAsync(host, d, cells(w) * sizeof(float), cudaMemcpyDeviceToHost, w->stream));
    HG_CUDA(cudaStreamSynchronize(w->stream));
    return HG_OK;
}

int hg_world_upload_device(hg_world* w, int field, const float* dev) {
    HG_CHECK_WORLD(w);
    if (!dev) return fail(HG_ERR_INVALID, "null device pointer");
    float* d = field_ptr(w, field);
    if (!d) return fail(HG_ERR_INVALID, "bad field id");
    DeviceGuard g(w->device);
    HG_CUDA(cudaMemcpyAsync(d, dev, cells(w) * sizeof(float), cudaMemcpyDeviceToDevice, w->stream));
    if (field == HG_FIELD_KS) w->ks_on = true;
    return HG_OK;
}

int hg_world_download_device(hg_world* w, int field, float* dev) {
    HG_CHECK_WORLD(w);
    if (!dev) return fail(HG_ERR_INVALID, "null device pointer");
    float* d = field_ptr(w, field);
    if (!d) return fail(HG_ERR_INVALID, "bad field id");
    DeviceGuard g(w->device);
    HG_CUDA(cudaMemcpyAsync(dev, d, cells(w) * sizeof(float), cudaMemcpyDeviceToDevice, w->stream));
    return HG_OK;
}

int hg_world_get_step(const hg_world* w, uint64_t* step) {
    HG_CHECK_WORLD(w);
    if (!step) return fail(HG_ERR_INVALID, "null output");
    *step = w->step;
    return HG_OK;
}

int hg_world_set_step(hg_world* w, uint64_t step) {
    HG_CHECK_WORLD(w);
    w->step = step;
    return HG_OK;
}

int hg_step(hg_world* w, int nsteps, int mode) {
    HG_CHECK_WORLD(w);
    if (nsteps < 0) return fail(HG_ERR_INVALID, "nsteps must be >= 0");
    if (mode != HG_MODE_PLAIN && mode != HG_MODE_FUSED) return fail(HG_ERR_INVALID, "bad mode");
    DeviceGuard g(w->device);
    StepConsts c = make_consts(w);
    cudaStream_t st = w->stream;
    auto swap = [&](int f) { float* t = w->cur[f]; w->cur[f] = w->alt[f]; w->alt[f] = t; };
    if (mode == HG_MODE_PLAIN) {
        for (int k = 0; k < nsteps; ++k) {
            RainStep r = make_rain(w, w->step + 1);
            if (r.active) launch_rain(c, r, w->cur[S_WATER], st);
            launch_flux(c, w->cur[S_ROCK], w->cur[S_WATER], w->cur[S_FL], w->cur[S_FR], w->cur[S_FT],
                        w->cur[S_FB], w->alt[S_WATER], w->alt[S_FL], w->alt[S_FR], w->alt[S_FT], w->alt[S_FB],
                        w->u, w->v, w->vz, st);
            swap(S_WATER); swap(S_FL); swap(S_FR); swap(S_FT); swap(S_FB);
            launch_erosion(c, w->u, w->v, w->vz, w->cur[S_ROCK], w->alt[S_ROCK], w->cur[S_SED], st);
            swap(S_ROCK);
            launch_sediment(c, w->u, w->v, w->cur[S_SED], w->alt[S_SED], w->cur[S_WATER], st);
            swap(S_SED);
            if (c.thermal) {
                launch_thermal_out(c, w->cur[S_ROCK], w->tc, w->td, st);
                launch_thermal_in(c, w->cur[S_ROCK], w->tc, w->td, w->alt[S_ROCK], st);
                swap(S_ROCK);
            }
            w->step += 1;
        }
    } else {
        int tx = 0, ty = 0;
        if (!pick_tile(w, tx, ty))
            return fail(HG_ERR_UNSUPPORTED, "fused mode needs n divisible by its 64x16 tile");
        for (int k = 0; k < nsteps; ++k) {
            FusedArgs a{};
            a.c = c;
            a.rain[0] = make_rain(w, w->step + 1);
            for (int f = 0; f < S_COUNT; ++f) { a.in.f[f] = w->cur[f]; a.out.f[f] = w->alt[f]; }
            a.u = w->u;
            a.v = w->v;
            a.s_ero = w->s_ero;
            a.b_ero = w->b_ero;
            a.err = w->err;
            if (!launch_fused(a, w->tma, st))
                return fail(HG_ERR_CUDA, "cuTensorMapEncodeTiled failed for a world buffer");
            for (int f = 0; f < S_COUNT; ++f) swap(f);
            w->step += 1;
        }
    }
    HG_CUDA(cudaGetLastError());
    return HG_OK;
}

int hg_sync(hg_world* w) {
    HG_CHECK_WORLD(w);
    DeviceGuard g(w->device);
    HG_CUDA(cudaStreamSynchronize(w->stream));
    int flag = 0;
    HG_CUDA(cudaMemcpy(&flag, w->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) {
        HG_CUDA(cudaMemset(w->err, 0, sizeof(int)));
        return fail(HG_ERR_TIMEOUT, "a fused-step tile load did not arrive within its bounded wait; "
                                    "the step's fields are not valid");
    }
    return HG_OK;
}

int hg_world_totals(hg_world* w, double out[3]) {
    HG_CHECK_WORLD(w);
    if (!out) return fail(HG_ERR_INVALID, "null output");
    DeviceGuard g(w->device);
    PtrList8 pl{};
    pl.p[0] = w->cur[S_ROCK];
    pl.p[1] = w->cur[S_WATER];
    pl.p[2] = w->cur[S_SED];
    int parts = reduction_parts();
    double* res = w->red_d + 8 * parts;
    launch_sum_f64(pl, 3, cells(w), w->red_d, parts, res, w->stream);
    HG_CUDA(cudaGetLastError());
    HG_CUDA(cudaMemcpyAsync(out, res, 3 * sizeof(double), cudaMemcpyDeviceToHost, w->stream));
    HG_CUDA(cudaStreamSynchronize(w->stream));
    return HG_OK;
}

}  // extern "C"
