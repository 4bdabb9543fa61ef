// Host side of the C ABI: worlds, settings, step sequencing, transfers.
//
// A world owns its device fields (FP32 structure-of-arrays, n*n floats each,
// double-buffered where a pass reads neighbours), one CUDA stream and a few
// reduction scratch buffers.  hg_step sequences the passes the way
// Erosion::dispatch_grid does (src/erosion.cpp:158-200), swapping buffer
// pointers where the reference swaps Tex_pair read/write textures.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <array>
#include <memory>
#include <mutex>
#include <new>
#include <vector>
#include <string>

#include <limits>

#include <nvtx3/nvToolsExt.h>

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

struct Plan;

// Fused-step variant chosen by the autotuner: tile height (16 or 8) and
// whether steps replay a captured two-step CUDA graph.
struct Tuning {
    int th = 0;  // 0: not tuned yet
    int graph = 0;
    double ms[4] = {};  // ms per step of (16, direct), (16, graph), (8, direct), (8, graph)
    int per_world = 0;  // batches: each world's own launches were faster than one table launch
    double ms_per_world = 0.0;
};

// Droplets and momentum map of a particle-mode world (hg_particles_init).
struct Particles {
    int count = 0;
    ParticleBufs b{};
    float* mom[2][4] = {};  // momentum map (x, y, z, w): current, alternate
    std::vector<void*> allocs;
    ~Particles() {
        for (void* p : allocs) cudaFree(p);
    }
};
}  // namespace hg

using namespace hg;

struct hg_world {
    int n = 0;
    int row_lo = 0, row_hi = 0;  // rows the per-pass kernels compute (hg_set_rows; all by default)
    int layers = 1;
    int device = 0;
    cudaStream_t stream = nullptr;
    hg_erosion_settings es{};
    hg_rain_settings rs{};
    hg_map_settings map{};
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
    float* dirt[2] = {};      // two-layer worlds: dirt (current, alternate)
    float* sdirt[2] = {};     // two-layer worlds: dirt sediment (current, alternate)
    float* s_ero = nullptr;  // fused step: eroded sediment of every cell
    float* b_ero = nullptr;  // fused step: eroded rock of every cell
    int* err = nullptr;      // device flag: a bounded wait gave up
    bool invalid = false;    // a sync saw that flag: fields undefined until re-initialised or loaded
    unsigned long long* d_step = nullptr;  // device copy of `step`, advanced by the fused kernels
    bool dev_step_valid = false;           // d_step == step
    uint64_t version = 1;                  // bumps whenever settings, options or Ks change
    TmaCache tma;
    hg::Plan* plans[2] = {};               // fused plans of this world alone, tile height 16 / 8
    hg::Tuning tuning;                     // autotuned fused-step variant
    float* red_f = nullptr;   // min/max partials + result
    double* red_d = nullptr;  // FP64 partials + result
    std::vector<hg_tape*> tapes;     // live tapes of this world (freed with it)
    hg::Particles* parts = nullptr;  // particle mode: droplets and momentum map
    float4* r_hm = nullptr;          // ray-marcher: packed heightmap texels
    float2* r_sed = nullptr;         // ray-marcher: packed sediment texels
    uint8_t* r_rgba = nullptr;       // hg_render: device image
    float* r_rgb = nullptr;
    size_t r_pixels = 0;             // capacity of r_rgba / r_rgb
};

namespace hg {
void release_tapes(hg_world* w);
}  // namespace hg

struct hg_batch {
    std::vector<hg_world*> worlds;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    int* err = nullptr;
    hg::Plan* plans[2] = {};
    hg::Tuning tuning;
};

namespace hg {
// A fused launch plan over one or more worlds: two descriptor tables in
// device memory (step direction cur -> alt and alt -> cur as of the build),
// the terrains' first tile indices, and lazily captured two-step graphs.
struct Plan {
    std::vector<hg_world*> worlds;
    int th = 16;
    int total = 0;  // tiles over all terrains
    std::vector<TerrainDesc> h_tab[2];  // per direction; a single world launches from these
    BatchParams* bp[2] = {};            // batch launches: terrain records (kernel parameter)
    CUtensorMap* d_maps[2] = {};        // batch launches: tensor maps in device memory
    std::vector<std::array<const float*, S_COUNT>> key_cur, key_alt;  // buffers at build time
    std::vector<float*> smooth_dst[2];  // per direction and world: the step's rock output when smoothing runs
                                        // (the fused kernels then leave their rock in the world's scratch)
    std::vector<uint64_t> versions;
    // captured steps starting with table 0 / table 1: [0] two steps, [1] kLongGraph
    cudaGraphExec_t graph[2][2] = {};
    uint64_t graph_launches[2] = {4, 4};  // kernel launches in one replay of each
    cudaStream_t stream = nullptr;
    int* err = nullptr;
};

void destroy_plan(Plan*& p) {
    if (!p) return;
    for (auto& gl : p->graph)
        for (auto& g : gl)
            if (g) cudaGraphExecDestroy(g);
    for (int d = 0; d < 2; ++d) {
        cudaFree(p->d_maps[d]);
        delete p->bp[d];
    }
    delete p;
    p = nullptr;
}
}  // namespace hg

namespace {

thread_local std::string t_err;

// The host log hook (hg_set_log_callback): set rarely, read on every
// report.  The (function, user) pair is published as one pointer to an
// immutable record, so a report never pairs a new function with an old
// user pointer; records stay alive until exit (a reader may still hold one).
struct LogHook {
    hg_log_fn fn;
    void* user;
};
std::atomic<const LogHook*> g_log{nullptr};
std::mutex g_log_mu;
std::vector<std::unique_ptr<LogHook>> g_log_hooks;  // every record ever published

void log_msg(int level, const std::string& msg) {
    if (const LogHook* h = g_log.load(std::memory_order_acquire))
        if (h->fn) h->fn(level, msg.c_str(), h->user);
}

int fail(int code, const std::string& msg) {
    t_err = msg;
    log_msg(HG_LOG_ERROR, msg);
    return code;
}

// NVTX range over an entry point (visible in Nsight timelines; header-only
// NVTX3, a no-op when no tool is attached)
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
};

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

// Entry points that advance or read a world's state refuse a world whose
// fields a timed-out tile load left undefined.
#define HG_CHECK_VALID(w)                                                                      \
    if ((w)->invalid)                                                                          \
    return fail(HG_ERR_TIMEOUT, "the world's fields are undefined after a timed-out tile load; " \
                                "re-initialise it (hg_init_heightmap, hg_init_reference_heightmap) or load it")

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
    for (int k = 0; k < 2; ++k) {
        cudaFree(w->dirt[k]);
        cudaFree(w->sdirt[k]);
    }
    cudaFree(w->s_ero); cudaFree(w->b_ero); cudaFree(w->err); cudaFree(w->d_step);
    for (Plan*& p : w->plans) destroy_plan(p);
    cudaFree(w->red_f); cudaFree(w->red_d);
    delete w->parts;
    w->parts = nullptr;
    cudaFree(w->r_hm); cudaFree(w->r_sed); cudaFree(w->r_rgba); cudaFree(w->r_rgb);
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

StepConsts make_consts(const hg_world* w);
// hg_set_rows restricted the per-pass kernels to a row slab: only one-layer
// per-pass steps and single passes honour it
bool rows_restricted(const hg_world* w) { return w->row_lo != 0 || w->row_hi != w->n; }
// the reversed step covers rain, flux, erosion and sediment transport
bool adjoint_covers(const hg_world* w) {
    return w->layers == 1 && make_consts(w).smooth_m == 0.0f && w->opt.rain_mode != HG_RAIN_REFERENCE;
}

StepConsts make_consts(const hg_world* w) {
    StepConsts c{};
    const hg_erosion_settings& s = w->es;
    volatile float dt = s.d_t;  // products rounded once, as the shaders do per cell
    c.n = w->n;
    c.row_lo = w->row_lo;
    c.row_hi = w->row_hi;
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
    // a marked drop is also > 0: fold that into the thresholds (the smallest
    // positive float is the first drop > 0)
    const float tiny = std::numeric_limits<float>::denorm_min();
    if (c.talus_x_cross < tiny) c.talus_x_cross = tiny;
    if (c.talus_b_diag < tiny) c.talus_b_diag = tiny;
    c.fast_div = !(c.talus_x_cross < 0x1p-30f) && !(c.talus_b_diag < 0x1p-30f);
    // smoothing weight, glsl/smoothing.glsl:74 (GLSL clamp: min(max(x, 0), 1))
    volatile float k1dt = s.Kspeed[1] * dt;
    float m = k1dt < 0.0f ? 0.0f : (float)k1dt;
    c.smooth_m = 1.0f < m ? 1.0f : m;
    c.Ks1 = s.Ks[1];
    c.Kconv = s.Kconv;
    c.Kalpha1 = s.Kalpha[1];
    c.Kspeed1 = s.Kspeed[1];
    return c;
}

Talus1 make_talus1(const hg_world* w) {
    Talus1 t{};
    t.x_cross = talus_cross_threshold(w->es.Kalpha[1]);
    t.b_diag = talus_diag_threshold(t.x_cross);
    const float tiny = std::numeric_limits<float>::denorm_min();
    if (t.x_cross < tiny) t.x_cross = tiny;
    if (t.b_diag < tiny) t.b_diag = tiny;
    t.fast_div = !(t.x_cross < 0x1p-30f) && !(t.b_diag < 0x1p-30f);
    return t;
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

RainBase make_rain_base(const hg_world* w) {
    RainStep r = make_rain(w, 1);
    RainBase b{};
    b.mode = w->opt.rain_mode;
    b.period = w->rs.period;
    b.amount = r.amount;
    b.threshold = r.threshold;
    b.seed_lo = r.seed_lo;
    b.seed_hi = r.seed_hi;
    b.terrain_id = r.terrain_id;
    return b;
}

__global__ void k_set_u64(unsigned long long* p, unsigned long long v) { *p = v; }

// frame time of step step1 for the reference rain
float rain_time(const hg_world* w, uint64_t step1) {
    return (float)((double)w->opt.rain_time0 + (double)step1 * (double)w->opt.rain_time_step);
}

// The rain pass of step step1 (1-based) on `water`, if it rains then.
void rain_pass(hg_world* w, const StepConsts& c, uint64_t step1, const float* rock, const float* dirt, float* water,
               cudaStream_t st) {
    RainStep r = make_rain(w, step1);
    if (!r.active) return;
    if (w->opt.rain_mode == HG_RAIN_REFERENCE)
        launch_ref_rain(w->rs, w->map, rain_time(w, step1), w->n, rock, dirt, water, st);
    else
        launch_rain(c, r, water, st);
}

// Fills both descriptor tables of a plan from its worlds' current buffers
// (table 0 steps cur -> alt, table 1 alt -> cur) and records the build state.
int build_plan(Plan* p) {
    const size_t nt = p->worlds.size();
    for (auto& gl : p->graph)  // captured launches hold the old descriptors
        for (auto& g : gl)
            if (g) {
                cudaStreamSynchronize(p->stream);
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
    std::vector<int> tile0(nt);
    p->total = 0;
    for (size_t i = 0; i < nt; ++i) {
        tile0[i] = p->total;
        p->total += fused_tiles(p->worlds[i]->n, p->th);
    }
    std::vector<TerrainDesc> tab(nt);
    for (int dir = 0; dir < 2; ++dir) {
        for (size_t i = 0; i < nt; ++i) {
            hg_world* w = p->worlds[i];
            TerrainSrc s{};
            s.c = make_consts(w);
            s.rain = make_rain_base(w);
            for (int f = 0; f < S_COUNT; ++f) {
                s.in[f] = dir == 0 ? w->cur[f] : w->alt[f];
                s.out[f] = dir == 0 ? w->alt[f] : w->cur[f];
            }
            s.u = w->u;
            s.v = w->v;
            s.s_ero = w->s_ero;
            s.b_ero = w->b_ero;
            s.step = w->d_step;
            p->smooth_dst[dir].resize(nt);
            p->smooth_dst[dir][i] = nullptr;
            if (s.c.smooth_m != 0.0f) {  // smoothing reads the fused rock from scratch into the real output
                p->smooth_dst[dir][i] = s.out[S_ROCK];
                s.out[S_ROCK] = reinterpret_cast<float*>(w->tc);
            }
            if (!fill_desc(tab[i], s, p->th, tile0[i], w->tma))
                return fail(HG_ERR_CUDA, "cuTensorMapEncodeTiled failed for a world buffer");
        }
        p->h_tab[dir] = tab;
        if (nt > 1) {  // batch: records as a kernel parameter, tensor maps in device memory
            if (!p->bp[dir]) p->bp[dir] = new BatchParams();
            BatchParams& bp = *p->bp[dir];
            bp.nterr = (int)nt;
            std::vector<CUtensorMap> maps(nt * MAPS_PER_TERRAIN);
            for (size_t i = 0; i < nt; ++i) {
                bp.tile0[i] = tile0[i];
                bp.t[i] = tab[i].h;
                for (int m = 0; m < MAPS_PER_TERRAIN; ++m) maps[i * MAPS_PER_TERRAIN + m] = tab[i].maps[m];
            }
            if (!p->d_maps[dir]) HG_CUDA(cudaMalloc((void**)&p->d_maps[dir], sizeof(CUtensorMap) * maps.size()));
            HG_CUDA(cudaMemcpyAsync(p->d_maps[dir], maps.data(), sizeof(CUtensorMap) * maps.size(),
                                    cudaMemcpyHostToDevice, p->stream));
            HG_CUDA(cudaStreamSynchronize(p->stream));  // `maps` is a local host buffer
        }
    }
    p->key_cur.resize(nt);
    p->key_alt.resize(nt);
    p->versions.resize(nt);
    for (size_t i = 0; i < nt; ++i) {
        for (int f = 0; f < S_COUNT; ++f) {
            p->key_cur[i][f] = p->worlds[i]->cur[f];
            p->key_alt[i][f] = p->worlds[i]->alt[f];
        }
        p->versions[i] = p->worlds[i]->version;
    }
    return HG_OK;
}

// Direction (table) of the next step: 0 if every world's current buffers are
// the build's cur, 1 if they are the build's alt, -1 if the plan is stale
// (settings changed, or per-pass steps swapped fields individually).
int plan_dir(const Plan* p) {
    if (p->key_cur.size() != p->worlds.size()) return -1;
    int dir = -1;
    for (size_t i = 0; i < p->worlds.size(); ++i) {
        const hg_world* w = p->worlds[i];
        if (w->version != p->versions[i]) return -1;
        bool is_cur = true, is_alt = true;
        for (int f = 0; f < S_COUNT; ++f) {
            is_cur = is_cur && w->cur[f] == p->key_cur[i][f];
            is_alt = is_alt && w->cur[f] == p->key_alt[i][f];
        }
        int d = is_cur ? 0 : is_alt ? 1 : -1;
        if (d < 0 || (dir >= 0 && d != dir)) return -1;
        dir = d;
    }
    return dir;
}

// One fused step in direction `dir`: a single world takes its descriptor as
// a kernel parameter, a batch launches over the device table.
void launch_dir(Plan* p, int dir) {
    if (p->worlds.size() == 1) launch_fused_one(p->h_tab[dir][0], p->th, p->err, p->stream);
    else launch_fused_table(*p->bp[dir], p->d_maps[dir], p->total, p->th, p->err, p->stream);
    // smoothing (worlds with Kspeed[1] != 0): the fused kernels left the
    // step's rock in scratch (the per-pass thermal buffer); the per-pass
    // smoothing kernel writes it into the step's rock output
    for (size_t i = 0; i < p->worlds.size(); ++i) {
        const TerrainHot& h = p->h_tab[dir][i].h;
        if (h.c.smooth_m == 0.0f) continue;
        launch_smooth(h.c, h.out[S_ROCK], p->smooth_dst[dir][i], p->stream);
    }
}

// Brings a plan up to date (tables, device step counters, the graph that
// starts with the next direction) without running a step; *dir gets the
// next direction.
// Steps per replay of a plan's long graph: long runs replay kLongGraph
// steps at a time (an even count: the buffers are back in their roles
// after it), a quarter of the host's graph launches.
constexpr int kLongGraph = 8;

// Captures (once) the graph of `which` (0: two steps, 1: kLongGraph steps)
// starting with descriptor table `dir`.
int capture_steps(Plan* p, int dir, int which) {
    if (p->graph[which][dir]) return HG_OK;
    const int steps = which ? kLongGraph : 2;
    cudaGraph_t g = nullptr;
    const uint64_t before = g_launches.load();
    HG_CUDA(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < steps; ++k) launch_dir(p, (dir + k) & 1);
    cudaError_t e = cudaStreamEndCapture(p->stream, &g);
    p->graph_launches[which] = g_launches.load() - before;  // captured, not run
    g_launches.fetch_sub(p->graph_launches[which]);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&p->graph[which][dir], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    return HG_OK;
}

int prepare_plan(Plan* p, bool use_graph, int* dir_out) {
    int dir = plan_dir(p);
    if (dir < 0) {
        int rc = build_plan(p);
        if (rc != HG_OK) return rc;
        dir = 0;
    }
    for (hg_world* w : p->worlds)
        if (!w->dev_step_valid) {
            k_set_u64<<<1, 1, 0, p->stream>>>(w->d_step, (unsigned long long)w->step);
            w->dev_step_valid = true;
        }
    if (use_graph)  // both lengths up front: no capture inside a later call's steps
        for (int which = 0; which < 2; ++which) {
            int rc = capture_steps(p, dir, which);
            if (rc != HG_OK) return rc;
        }
    *dir_out = dir;
    return HG_OK;
}

// Runs nsteps fused steps of a plan's worlds on the plan's stream.
int run_plan(Plan* p, int nsteps, bool use_graph) {
    // the reference rain runs as its own kernel before the steps it falls on,
    // so a plan with such a world launches step by step
    bool ref_rain = false;
    for (hg_world* w : p->worlds) ref_rain = ref_rain || w->opt.rain_mode == HG_RAIN_REFERENCE;
    if (ref_rain) use_graph = false;
    int dir = 0;
    int rc = prepare_plan(p, use_graph && nsteps >= 2, &dir);
    if (rc != HG_OK) return rc;
    const int nt = (int)p->worlds.size();
    int k = 0;
    if (use_graph && nsteps >= 2) {
        for (; k + kLongGraph <= nsteps; k += kLongGraph) {
            HG_CUDA(cudaGraphLaunch(p->graph[1][dir], p->stream));
            count_launch(p->graph_launches[1]);
        }
        for (; k + 2 <= nsteps; k += 2) {
            HG_CUDA(cudaGraphLaunch(p->graph[0][dir], p->stream));
            count_launch(p->graph_launches[0]);
        }
    }
    for (; k < nsteps; ++k) {
        const int d = (dir + k) & 1;
        if (ref_rain)  // the step's input water: the buffers of direction d at the plan's build
            for (int i = 0; i < nt; ++i) {
                hg_world* w = p->worlds[i];
                if (w->opt.rain_mode != HG_RAIN_REFERENCE) continue;
                const auto& in = d == 0 ? p->key_cur[i] : p->key_alt[i];
                rain_pass(w, StepConsts{}, w->step + (uint64_t)k + 1, in[S_ROCK], nullptr,
                          const_cast<float*>(in[S_WATER]), p->stream);
            }
        launch_dir(p, d);
    }
    HG_CUDA(cudaGetLastError());
    for (hg_world* w : p->worlds) {
        w->step += (uint64_t)nsteps;
        if (nsteps & 1)
            for (int f = 0; f < S_COUNT; ++f) std::swap(w->cur[f], w->alt[f]);
    }
    return HG_OK;
}

// Fused steps over `worlds` with the autotuned (or requested) variant.  The
// first call with at least 8 steps and no tuned choice times two steps of
// each variant (tile height 16/8 x direct launches/graph replay); every
// variant gives identical fields, so tuning steps are ordinary steps.  Graph
// replay runs kLongGraph steps per replay while that many remain, then two.
int fused_run(Plan** plans, const std::vector<hg_world*>& worlds, Tuning& tune, int req_th, int req_graph,
              cudaStream_t st, int* err, int nsteps) {
    for (hg_world* w : worlds) {
        if (!fused_tile_ok(w->n, 16)) return fail(HG_ERR_UNSUPPORTED, "fused mode needs n divisible by 64");
        if (w->layers != 1) return fail(HG_ERR_UNSUPPORTED, "the fused step covers one-layer worlds");
    }
    if (req_th != HG_AUTO && req_th != 16 && req_th != 8)
        return fail(HG_ERR_UNSUPPORTED, "fused tile height must be 16 or 8");
    auto plan_for = [&](int th) -> Plan* {
        Plan*& p = plans[th == 16 ? 0 : 1];
        if (!p) {
            p = new Plan();
            p->worlds = worlds;
            p->th = th;
            p->stream = st;
            p->err = err;
        }
        return p;
    };
    if (req_th == HG_AUTO && req_graph == HG_AUTO && tune.th == 0 && nsteps >= 8) {
        cudaEvent_t e0, e1;
        HG_CUDA(cudaEventCreate(&e0));
        HG_CUDA(cudaEventCreate(&e1));
        double best = 1e30;
        for (int cand = 0; cand < 4; ++cand) {
            int th = cand < 2 ? 16 : 8, graph = cand & 1;
            int dir = 0;
            int rc0 = prepare_plan(plan_for(th), graph != 0, &dir);  // host work outside the timed span
            if (rc0 != HG_OK) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc0; }
            cudaEventRecord(e0, st);
            int rc = run_plan(plan_for(th), 2, graph != 0);
            cudaEventRecord(e1, st);
            if (rc != HG_OK) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
            HG_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            tune.ms[cand] = ms / 2.0;
            if (tune.ms[cand] < best) { best = tune.ms[cand]; tune.th = th; tune.graph = graph; }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        nsteps -= 8;
        char m[160];
        std::snprintf(m, sizeof m, "autotuner: %zu world(s), tile 64x%d, graph %s (ms/step: %.4f %.4f %.4f %.4f)",
                      worlds.size(), tune.th, tune.graph ? "on" : "off", tune.ms[0], tune.ms[1], tune.ms[2],
                      tune.ms[3]);
        log_msg(HG_LOG_INFO, m);
    }
    int th = req_th != HG_AUTO ? req_th : (tune.th ? tune.th : 16);
    int graph = req_graph != HG_AUTO ? req_graph : (tune.th ? tune.graph : 1);
    return run_plan(plan_for(th), nsteps, graph != 0);
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
        case HG_FIELD_DIRT: return w->dirt[0];
        case HG_FIELD_SEDIMENT_DIRT: return w->sdirt[0];
        case HG_FIELD_MOMENTUM_X: return w->parts ? w->parts->mom[0][0] : nullptr;
        case HG_FIELD_MOMENTUM_Y: return w->parts ? w->parts->mom[0][1] : nullptr;
    }
    return nullptr;
}

}  // namespace

int hg::hg_report_error(int code, const char* msg) { return fail(code, msg); }

extern "C" {

const char* hg_version(void) { return "hydrogen-gb300 0.1 (sm_103a)"; }
const char* hg_last_error(void) { return t_err.c_str(); }

int hg_set_log_callback(hg_log_fn fn, void* user) {
    std::lock_guard<std::mutex> lk(g_log_mu);
    g_log_hooks.push_back(std::unique_ptr<LogHook>(new LogHook{fn, user}));
    g_log.store(fn ? g_log_hooks.back().get() : nullptr, std::memory_order_release);
    return HG_OK;
}
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

int hg_default_particle_settings(hg_erosion_settings* out) {
    if (!out) return fail(HG_ERR_INVALID, "null settings");
    std::memset(out, 0, sizeof(*out));
    // particle-model defaults, src/state.cpp:61-79 (particle_count left at 0)
    out->Kc = 0.2f;
    out->Kalpha[0] = 1.3f; out->Kalpha[1] = 0.6f;
    out->Kconv = 0.001f;
    out->Ks[0] = 0.03f; out->Ks[1] = 0.09f;
    out->Kd[0] = 0.01f; out->Kd[1] = 0.03f;
    out->Ke = 0.03f;
    out->Kspeed[0] = 0.002f; out->Kspeed[1] = 0.008f;
    out->G = 9.81f;
    out->d_t = 0.25f;
    out->density = 1.0f;
    out->init_volume = 1.0f;
    out->friction = 0.2f;
    out->inertia = 1.0f;
    out->min_volume = 0.0f;
    out->min_velocity = 0.001f;
    out->ttl = 15000;
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
    out->graph = HG_AUTO;
    out->tile_x = HG_AUTO;
    out->tile_y = HG_AUTO;
    return HG_OK;
}

int hg_world_create(int n, int layers, hg_world** out) {
    if (!out) return fail(HG_ERR_INVALID, "null output pointer");
    *out = nullptr;
    if (n <= 0 || n % 8 != 0) return fail(HG_ERR_INVALID, "n must be a positive multiple of 8");
    if (layers != 1 && layers != 2) return fail(HG_ERR_UNSUPPORTED, "layers must be 1 or 2");
    hg_world* w = new (std::nothrow) hg_world();
    if (!w) return fail(HG_ERR_OOM, "host allocation failed");
    w->n = n;
    w->row_hi = n;
    w->layers = layers;
    cudaGetDevice(&w->device);
    hg_default_erosion_settings(&w->es);
    if (layers == 1) {
        w->es.Kconv = 0.0f;       // one-layer world: no dirt layer to convert into
        w->es.Kspeed[1] = 0.0f;
    }
    hg_default_rain_settings(&w->rs);
    hg_default_map_settings(&w->map);
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
    for (int k = 0; k < 2 && layers == 2 && e == cudaSuccess; ++k) {
        e = alloc((void**)&w->dirt[k], bytes);
        if (e == cudaSuccess) e = alloc((void**)&w->sdirt[k], bytes);
        if (e == cudaSuccess) e = cudaMemsetAsync(w->dirt[k], 0, bytes, w->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(w->sdirt[k], 0, bytes, w->stream);
    }
    if (e == cudaSuccess) e = alloc((void**)&w->s_ero, bytes);
    if (e == cudaSuccess) e = alloc((void**)&w->b_ero, bytes);
    if (e == cudaSuccess) e = alloc((void**)&w->err, sizeof(int));
    if (e == cudaSuccess) e = alloc((void**)&w->d_step, sizeof(unsigned long long));
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
    release_tapes(w);
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
    if (s->particle_count != 0 && (!w->parts || s->particle_count != (uint32_t)w->parts->count))
        return fail(HG_ERR_INVALID, "particle_count must be 0 or the droplet count of hg_particles_init");
    if (!(s->d_t > 0.0f) || !std::isfinite(s->d_t)) return fail(HG_ERR_INVALID, "d_t must be positive and finite");
    if (w->layers == 1 && s->Kconv != 0.0f)
        return fail(HG_ERR_INVALID, "Kconv must be 0 in a one-layer world (no dirt layer)");
    w->es = *s;
    w->version += 1;
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
    w->version += 1;
    return HG_OK;
}

int hg_set_step_options(hg_world* w, const hg_step_options* o) {
    HG_CHECK_WORLD(w);
    if (!o) return fail(HG_ERR_INVALID, "null options");
    if (o->rain_mode < HG_RAIN_OFF || o->rain_mode > HG_RAIN_REFERENCE) return fail(HG_ERR_INVALID, "bad rain_mode");
    if (!(o->rain_probability >= 0.0f && o->rain_probability <= 1.0f))
        return fail(HG_ERR_INVALID, "rain_probability must be in [0, 1]");
    if (o->tile_x != HG_AUTO && o->tile_x != 64) return fail(HG_ERR_UNSUPPORTED, "fused tile width must be 64");
    if (o->tile_y != HG_AUTO && o->tile_y != 16 && o->tile_y != 8)
        return fail(HG_ERR_UNSUPPORTED, "fused tile height must be 16 or 8");
    if (o->graph != HG_AUTO && o->graph != 0 && o->graph != 1) return fail(HG_ERR_INVALID, "graph must be -1, 0 or 1");
    w->opt = *o;
    w->version += 1;
    return HG_OK;
}

namespace {
// idle droplets, zero momentum map
int reset_particles(hg_world* w) {
    Particles& P = *w->parts;
    const size_t cnt = (size_t)P.count, bytes = cells(w) * sizeof(float);
    const Drops& d = P.b.d;
    for (float* f : {d.px, d.py, d.vx, d.vy, d.vol, d.s0, d.s1, d.sc})
        HG_CUDA(cudaMemsetAsync(f, 0, cnt * sizeof(float), w->stream));
    HG_CUDA(cudaMemsetAsync(d.iters, 0, cnt * sizeof(uint32_t), w->stream));
    HG_CUDA(cudaMemsetAsync(d.kill, 0, cnt * sizeof(int32_t), w->stream));
    for (int k = 0; k < 2; ++k)
        for (int c = 0; c < 4; ++c) HG_CUDA(cudaMemsetAsync(P.mom[k][c], 0, bytes, w->stream));
    return HG_OK;
}

// every state field (and the dirt layer's) back to zero
int zero_state(hg_world* w) {
    size_t bytes = cells(w) * sizeof(float);
    for (int f = 0; f < S_COUNT; ++f) {
        HG_CUDA(cudaMemsetAsync(w->cur[f], 0, bytes, w->stream));
        HG_CUDA(cudaMemsetAsync(w->alt[f], 0, bytes, w->stream));
    }
    HG_CUDA(cudaMemsetAsync(w->u, 0, bytes, w->stream));
    HG_CUDA(cudaMemsetAsync(w->v, 0, bytes, w->stream));
    HG_CUDA(cudaMemsetAsync(w->vz, 0, bytes, w->stream));
    for (int k = 0; k < 2 && w->layers == 2; ++k) {
        HG_CUDA(cudaMemsetAsync(w->dirt[k], 0, bytes, w->stream));
        HG_CUDA(cudaMemsetAsync(w->sdirt[k], 0, bytes, w->stream));
    }
    if (w->parts) return reset_particles(w);
    return HG_OK;
}

int check_map_settings(const hg_map_settings* s) {
    if (!s) return fail(HG_ERR_INVALID, "null map settings");
    if (s->octaves < 0) return fail(HG_ERR_INVALID, "octaves must be >= 0");
    if (!(s->max_height > 0.0f)) return fail(HG_ERR_INVALID, "max_height must be positive");
    return HG_OK;
}
}  // namespace

int hg_default_map_settings(hg_map_settings* out) {
    if (!out) return fail(HG_ERR_INVALID, "null settings");
    std::memset(out, 0, sizeof(*out));
    // src/settings.hpp:27-57 (MAX_HEIGHT 256, WATER_HEIGHT 96)
    out->max_height = 256.0f;
    out->max_dirt = 2.0f;
    out->hmap_dims[0] = out->hmap_dims[1] = 1024;
    out->height_mult = 1.0f;
    out->water_lvl = 96.0f;
    out->seed = 0.0f;
    out->persistance = 0.44f;
    out->lacunarity = 2.0f;
    out->scale = 0.00075f;
    out->redistribution = 1.0f;
    out->octaves = 8;
    out->mask_exp = 1;
    out->mask_power = 1;
    out->uplift_scale = 1.16f;
    out->domain_warp = 1;
    out->domain_warp_scale = 100.0f;
    out->terrace_scale = 0.5f;
    return HG_OK;
}

int hg_set_map_settings(hg_world* w, const hg_map_settings* s) {
    HG_CHECK_WORLD(w);
    int rc = check_map_settings(s);
    if (rc != HG_OK) return rc;
    w->map = *s;
    w->version += 1;
    return HG_OK;
}

int hg_init_reference_heightmap(hg_world* w, const hg_map_settings* s) {
    Range nv_range("hg_init_reference_heightmap");
    HG_CHECK_WORLD(w);
    int rc = check_map_settings(s);
    if (rc != HG_OK) return rc;
    DeviceGuard g(w->device);
    if ((rc = zero_state(w)) != HG_OK) return rc;
    launch_ref_heightmap(*s, w->n, w->cur[S_ROCK], w->layers == 2 ? w->dirt[0] : nullptr, w->stream);
    HG_CUDA(cudaGetLastError());
    w->map = *s;
    w->version += 1;
    w->step = 0;
    w->dev_step_valid = false;
    w->invalid = false;
    return HG_OK;
}

int hg_camera_look_at(hg_camera* out, const float pos[3], const float dir[3], const float up[3], float fov_deg,
                      float aspect, float z_near, float z_far) {
    if (!out || !pos || !dir || !up) return fail(HG_ERR_INVALID, "null argument");
    if (!(aspect > 0.0f) || !(z_far > z_near) || !(fov_deg > 0.0f && fov_deg < 180.0f))
        return fail(HG_ERR_INVALID, "bad projection");
    std::memset(out, 0, sizeof(*out));
    auto norm = [](float v[3]) {
        const float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        v[0] /= l; v[1] /= l; v[2] /= l;
    };
    auto cross = [](const float a[3], const float b[3], float r[3]) {
        r[0] = a[1] * b[2] - b[1] * a[2];
        r[1] = a[2] * b[0] - b[2] * a[0];
        r[2] = a[0] * b[1] - b[0] * a[1];
    };
    auto dot = [](const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    // lookAt(eye = pos, center = pos + dir, up), right-handed
    float f[3] = {(pos[0] + dir[0]) - pos[0], (pos[1] + dir[1]) - pos[1], (pos[2] + dir[2]) - pos[2]};
    norm(f);
    float s[3], u[3];
    cross(f, up, s);
    norm(s);
    cross(s, f, u);
    float* V = out->view;
    V[0] = s[0]; V[4] = s[1]; V[8] = s[2];
    V[1] = u[0]; V[5] = u[1]; V[9] = u[2];
    V[2] = -f[0]; V[6] = -f[1]; V[10] = -f[2];
    V[12] = -dot(s, pos); V[13] = -dot(u, pos); V[14] = dot(f, pos);
    V[15] = 1.0f;
    // perspective, depth -1..1
    const float th = std::tan(fov_deg * 0.01745329251994329577f / 2.0f);
    float* P = out->perspective;
    P[0] = 1.0f / (aspect * th);
    P[5] = 1.0f / th;
    P[10] = -(z_far + z_near) / (z_far - z_near);
    P[11] = -1.0f;
    P[14] = -(2.0f * z_far * z_near) / (z_far - z_near);
    for (int k = 0; k < 3; ++k) out->pos[k] = pos[k];
    out->prec = 0.35f;
    out->draw_water = 1;
    out->display_sediment = 0;
    out->sediment_max_cap = 0.1f;
    out->low_res_div3 = 0;
    return HG_OK;
}

int hg_render_device(hg_world* w, const hg_camera* cam, int width, int height, uint8_t* rgba_dev, float* rgb_dev) {
    Range nv_range("hg_render_device");
    HG_CHECK_WORLD(w);
    if (!cam || !rgba_dev) return fail(HG_ERR_INVALID, "null argument");
    if (width < 1 || height < 1 || (size_t)width * height > (size_t)1 << 28)
        return fail(HG_ERR_INVALID, "image size must be in [1, 2^28] pixels");
    if (!(cam->prec > 0.0f) || !std::isfinite(cam->prec)) return fail(HG_ERR_INVALID, "prec must be positive");
    DeviceGuard g(w->device);
    const size_t bytes = cells(w);
    if (!w->r_hm) HG_CUDA(cudaMalloc((void**)&w->r_hm, bytes * sizeof(float4)));
    if (cam->display_sediment && !w->r_sed) HG_CUDA(cudaMalloc((void**)&w->r_sed, bytes * sizeof(float2)));
    RenderInput in{w->n, w->map.max_height, w->map.hmap_dims[0], w->cur[S_ROCK], w->layers == 2 ? w->dirt[0] : nullptr,
                   w->cur[S_WATER], w->cur[S_SED], w->layers == 2 ? w->sdirt[0] : nullptr, w->r_hm, w->r_sed};
    int rc = render_image(in, *cam, width, height, rgba_dev, rgb_dev, w->stream);
    if (rc != HG_OK) return fail(rc, "singular view or perspective matrix");
    HG_CUDA(cudaGetLastError());
    return HG_OK;
}

int hg_render(hg_world* w, const hg_camera* cam, int width, int height, uint8_t* rgba, float* rgb) {
    Range nv_range("hg_render");
    HG_CHECK_WORLD(w);
    if (!cam || !rgba) return fail(HG_ERR_INVALID, "null argument");
    if (width < 1 || height < 1 || (size_t)width * height > (size_t)1 << 28)
        return fail(HG_ERR_INVALID, "image size must be in [1, 2^28] pixels");
    DeviceGuard g(w->device);
    const size_t px = (size_t)width * height;
    if (px > w->r_pixels) {
        cudaFree(w->r_rgba);
        cudaFree(w->r_rgb);
        w->r_rgba = nullptr;
        w->r_rgb = nullptr;
        w->r_pixels = 0;
        HG_CUDA(cudaMalloc((void**)&w->r_rgba, px * 4));
        HG_CUDA(cudaMalloc((void**)&w->r_rgb, px * 3 * sizeof(float)));
        w->r_pixels = px;
    }
    int rc = hg_render_device(w, cam, width, height, w->r_rgba, rgb ? w->r_rgb : nullptr);
    if (rc != HG_OK) return rc;
    HG_CUDA(cudaMemcpyAsync(rgba, w->r_rgba, px * 4, cudaMemcpyDeviceToHost, w->stream));
    if (rgb) HG_CUDA(cudaMemcpyAsync(rgb, w->r_rgb, px * 3 * sizeof(float), cudaMemcpyDeviceToHost, w->stream));
    HG_CUDA(cudaStreamSynchronize(w->stream));
    return HG_OK;
}

int hg_rain(hg_world* w, float time) {
    HG_CHECK_WORLD(w);
    HG_CHECK_VALID(w);
    DeviceGuard g(w->device);
    if (w->opt.rain_mode == HG_RAIN_OFF) return HG_OK;
    if (w->opt.rain_mode == HG_RAIN_REFERENCE) {
        launch_ref_rain(w->rs, w->map, time, w->n, w->cur[S_ROCK], w->layers == 2 ? w->dirt[0] : nullptr,
                        w->cur[S_WATER], w->stream);
    } else {
        RainStep r = make_rain(w, w->step + 1);
        r.active = 1;
        launch_rain(make_consts(w), r, w->cur[S_WATER], w->stream);
    }
    HG_CUDA(cudaGetLastError());
    return HG_OK;
}

int hg_particles_init(hg_world* w, int count) {
    HG_CHECK_WORLD(w);
    if (w->layers != 2) return fail(HG_ERR_UNSUPPORTED, "particle erosion runs on two-layer worlds");
    if (count < 1 || count > (1 << 28)) return fail(HG_ERR_INVALID, "count must be in [1, 2^28]");
    DeviceGuard g(w->device);
    HG_CUDA(cudaStreamSynchronize(w->stream));
    delete w->parts;
    w->parts = nullptr;
    Particles* P = new (std::nothrow) Particles();
    if (!P) return fail(HG_ERR_OOM, "host allocation failed");
    const size_t cnt = (size_t)count, cl = cells(w);
    cudaError_t e = cudaSuccess;
    auto take = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (e == cudaSuccess) e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) P->allocs.push_back(p);
        return e == cudaSuccess ? p : nullptr;
    };
    Drops& d = P->b.d;
    d.count = count;
    float** fs[8] = {&d.px, &d.py, &d.vx, &d.vy, &d.vol, &d.s0, &d.s1, &d.sc};
    for (float** f : fs) *f = (float*)take(cnt * sizeof(float));
    d.iters = (uint32_t*)take(cnt * sizeof(uint32_t));
    d.kill = (int32_t*)take(cnt * sizeof(int32_t));
    P->b.cnt = (uint32_t*)take(cl * sizeof(uint32_t));
    P->b.offs = (uint32_t*)take((cl + 1) * sizeof(uint32_t));
    P->b.cursor = (uint32_t*)take(cl * sizeof(uint32_t));
    P->b.block_sums = (uint32_t*)take(particle_scan_blocks(cl) * sizeof(uint32_t));
    P->b.keys = (uint32_t*)take(4 * cnt * sizeof(uint32_t));
    P->b.sorted = (uint32_t*)take(4 * cnt * sizeof(uint32_t));
    P->b.hot_cap = (uint32_t)particle_hot_capacity(cl, count);
    P->b.hot = (uint32_t*)take((2 + 2 * (size_t)P->b.hot_cap) * sizeof(uint32_t));
    P->b.rec = (float*)take(8 * cnt * sizeof(float));
    P->b.rec_mask = (uint8_t*)take(4 * cnt);
    for (int k = 0; k < 2; ++k)
        for (int c = 0; c < 4; ++c) P->mom[k][c] = (float*)take(cl * sizeof(float));
    if (e != cudaSuccess) {
        delete P;
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? HG_ERR_OOM : HG_ERR_CUDA,
                    std::string("particle allocation: ") + cudaGetErrorString(e));
    }
    P->count = count;
    w->parts = P;
    int rc = reset_particles(w);
    if (rc != HG_OK) return rc;
    HG_CUDA(cudaStreamSynchronize(w->stream));
    return HG_OK;
}

int hg_particles_get(hg_world* w, float* state8, uint32_t* iters, int32_t* kill) {
    HG_CHECK_WORLD(w);
    if (!w->parts) return fail(HG_ERR_INVALID, "no droplets: call hg_particles_init first");
    DeviceGuard g(w->device);
    const Drops& d = w->parts->b.d;
    const size_t cnt = (size_t)d.count;
    if (state8) {
        std::vector<float> col(cnt);
        const float* fs[8] = {d.px, d.py, d.vx, d.vy, d.vol, d.s0, d.s1, d.sc};
        for (int k = 0; k < 8; ++k) {
            HG_CUDA(cudaMemcpyAsync(col.data(), fs[k], cnt * sizeof(float), cudaMemcpyDeviceToHost, w->stream));
            HG_CUDA(cudaStreamSynchronize(w->stream));
            for (size_t i = 0; i < cnt; ++i) state8[8 * i + k] = col[i];
        }
    }
    if (iters) HG_CUDA(cudaMemcpyAsync(iters, d.iters, cnt * sizeof(uint32_t), cudaMemcpyDeviceToHost, w->stream));
    if (kill) HG_CUDA(cudaMemcpyAsync(kill, d.kill, cnt * sizeof(int32_t), cudaMemcpyDeviceToHost, w->stream));
    HG_CUDA(cudaStreamSynchronize(w->stream));
    return HG_OK;
}

int hg_particles_count(const hg_world* w, int* count) {
    HG_CHECK_WORLD(w);
    if (!count) return fail(HG_ERR_INVALID, "null output");
    *count = w->parts ? w->parts->count : 0;
    return HG_OK;
}

int hg_init_heightmap(hg_world* w, const hg_noise_settings* s) {
    Range nv_range("hg_init_heightmap");
    HG_CHECK_WORLD(w);
    if (!s) return fail(HG_ERR_INVALID, "null noise settings");
    if (s->octaves < 1 || s->octaves > 32) return fail(HG_ERR_INVALID, "octaves must be in [1, 32]");
    DeviceGuard g(w->device);
    int zrc = zero_state(w);
    if (zrc != HG_OK) return zrc;
    launch_fbm_raw(w->cur[S_ROCK], w->n, *s, w->stream);
    launch_minmax(w->cur[S_ROCK], cells(w), w->red_f, reduction_parts(), w->red_f + 2 * reduction_parts(),
                  w->stream);
    launch_scale(w->cur[S_ROCK], cells(w), w->red_f + 2 * reduction_parts(), s->out_min, s->out_max, w->stream);
    HG_CUDA(cudaGetLastError());
    w->step = 0;
    w->dev_step_valid = false;
    w->invalid = false;
    return HG_OK;
}

int hg_init_heightmap_host(hg_world* w, const float* rock) {
    Range nv_range("hg_init_heightmap_host");
    HG_CHECK_WORLD(w);
    if (!rock) return fail(HG_ERR_INVALID, "null heightmap");
    DeviceGuard g(w->device);
    int rc = zero_state(w);
    if (rc != HG_OK) return rc;
    HG_CUDA(cudaMemcpyAsync(w->cur[S_ROCK], rock, cells(w) * sizeof(float), cudaMemcpyHostToDevice, w->stream));
    HG_CUDA(cudaStreamSynchronize(w->stream));
    w->step = 0;
    w->dev_step_valid = false;
    w->invalid = false;
    return HG_OK;
}

int hg_world_count_nonfinite(hg_world* w, uint64_t* count) {
    HG_CHECK_WORLD(w);
    if (!count) return fail(HG_ERR_INVALID, "null output");
    DeviceGuard g(w->device);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(w->red_d);  // 8 bytes of reduction scratch
    HG_CUDA(cudaMemsetAsync(d, 0, sizeof(*d), w->stream));
    const size_t c = cells(w);
    for (int f = 0; f < S_COUNT; ++f) launch_count_nonfinite(w->cur[f], c, d, w->stream);
    launch_count_nonfinite(w->u, c, d, w->stream);
    launch_count_nonfinite(w->v, c, d, w->stream);
    if (w->layers == 2) {
        launch_count_nonfinite(w->dirt[0], c, d, w->stream);
        launch_count_nonfinite(w->sdirt[0], c, d, w->stream);
    }
    if (w->parts) {  // the momentum map and every droplet's float state
        const Particles& P = *w->parts;
        for (int ch = 0; ch < 4; ++ch) launch_count_nonfinite(P.mom[0][ch], c, d, w->stream);
        const Drops& dr = P.b.d;
        for (float* f : {dr.px, dr.py, dr.vx, dr.vy, dr.vol, dr.s0, dr.s1, dr.sc})
            launch_count_nonfinite(f, (size_t)P.count, d, w->stream);
    }
    HG_CUDA(cudaGetLastError());
    unsigned long long h = 0;
    HG_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, w->stream));
    HG_CUDA(cudaStreamSynchronize(w->stream));
    *count = h;
    return HG_OK;
}

int hg_world_poison_scratch(hg_world* w) {
    HG_CHECK_WORLD(w);
    DeviceGuard g(w->device);
    const size_t b = cells(w) * sizeof(float);
    for (int f = 0; f < S_COUNT; ++f) HG_CUDA(cudaMemsetAsync(w->alt[f], 0xFF, b, w->stream));
    // u and v are carried (and counted) but belong to the grid step: a world
    // with droplets keeps them, since the particle step neither reads nor
    // writes them
    for (float* p : {w->parts ? nullptr : w->u, w->parts ? nullptr : w->v, w->vz, w->s_ero, w->b_ero, w->dirt[1],
                     w->sdirt[1]})
        if (p) HG_CUDA(cudaMemsetAsync(p, 0xFF, b, w->stream));
    for (float4* p : {w->tc, w->td})
        if (p) HG_CUDA(cudaMemsetAsync(p, 0xFF, 4 * b, w->stream));
    if (w->parts) {
        // the droplet records' sediment and layer mask (every record of a
        // moving droplet writes both before the replay reads them); the
        // momentum map's alternate is not scratch: border texels keep it
        // from two steps back, as the reference's ping-pong does
        const Particles& P = *w->parts;
        HG_CUDA(cudaMemsetAsync(P.b.rec, 0xFF, 8 * (size_t)P.count * sizeof(float), w->stream));
        HG_CUDA(cudaMemsetAsync(P.b.rec_mask, 0xFF, 4 * (size_t)P.count, w->stream));
    }
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
    w->version += 1;
    return HG_OK;
}

int hg_clear_ks_field(hg_world* w) {
    HG_CHECK_WORLD(w);
    w->ks_on = false;
    w->version += 1;
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
    if (field == HG_FIELD_KS) {
        w->ks_on = true;
        w->version += 1;
    }
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
    if (field == HG_FIELD_KS) {
        w->ks_on = true;
        w->version += 1;
    }
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
    w->dev_step_valid = false;
    return HG_OK;
}

namespace {
// Fused steps of a two-layer world: three kernels per step (hg_fused2.cu);
// the reference rain runs as its own kernel before the step it falls on.
int fused2_steps(hg_world* w, int nsteps) {
    if (!fused2_ok(w->n)) return fail(HG_ERR_UNSUPPORTED, "fused mode needs n divisible by 64");
    const StepConsts c = make_consts(w);
    const Talus1 t1 = make_talus1(w);
    cudaStream_t st = w->stream;
    const size_t cl = cells(w);
    float* scratch = reinterpret_cast<float*>(w->tc);  // 4 n^2 floats
    for (int k = 0; k < nsteps; ++k) {
        const uint64_t step1 = w->step + 1;
        RainStep r = make_rain(w, step1);
        if (w->opt.rain_mode == HG_RAIN_REFERENCE) {
            rain_pass(w, c, step1, w->cur[S_ROCK], w->dirt[0], w->cur[S_WATER], st);
            r.active = 0;
        }
        Fused2Bufs b{};
        b.rock = w->cur[S_ROCK]; b.dirt = w->dirt[0]; b.water = w->cur[S_WATER];
        b.s0 = w->cur[S_SED]; b.s1 = w->sdirt[0];
        b.fl = w->cur[S_FL]; b.fr = w->cur[S_FR]; b.ft = w->cur[S_FT]; b.fb = w->cur[S_FB];
        b.rock_o = w->alt[S_ROCK]; b.dirt_o = w->dirt[1]; b.water_o = w->alt[S_WATER];
        b.s0_o = w->alt[S_SED]; b.s1_o = w->sdirt[1];
        b.fl_o = w->alt[S_FL]; b.fr_o = w->alt[S_FR]; b.ft_o = w->alt[S_FT]; b.fb_o = w->alt[S_FB];
        b.u = w->u; b.v = w->v;
        b.s0_ero = w->s_ero; b.s1_ero = scratch; b.b_ero = w->b_ero;
        b.rock_mid = scratch + cl; b.g_ero = scratch + 2 * cl;
        int rc = launch_fused2_step(c, t1, r, b, w->tma, w->err, st);
        if (rc != HG_OK) return fail(rc, "cuTensorMapEncodeTiled failed for a world buffer");
        for (int f = 0; f < S_COUNT; ++f) std::swap(w->cur[f], w->alt[f]);
        std::swap(w->dirt[0], w->dirt[1]);
        std::swap(w->sdirt[0], w->sdirt[1]);
        w->step += 1;
    }
    w->dev_step_valid = false;
    HG_CUDA(cudaGetLastError());
    return HG_OK;
}
}  // namespace

int hg_step(hg_world* w, int nsteps, int mode) {
    Range nv_range("hg_step");
    HG_CHECK_WORLD(w);
    HG_CHECK_VALID(w);
    if (nsteps < 0) return fail(HG_ERR_INVALID, "nsteps must be >= 0");
    if (mode != HG_MODE_PLAIN && mode != HG_MODE_FUSED && mode != HG_MODE_PARTICLES)
        return fail(HG_ERR_INVALID, "bad mode");
    if (rows_restricted(w) && (mode != HG_MODE_PLAIN || w->layers != 1))
        return fail(HG_ERR_UNSUPPORTED, "a row-restricted world steps with the one-layer per-pass kernels only");
    DeviceGuard g(w->device);
    StepConsts c = make_consts(w);
    cudaStream_t st = w->stream;
    auto swap = [&](int f) { float* t = w->cur[f]; w->cur[f] = w->alt[f]; w->alt[f] = t; };
    if (mode == HG_MODE_PARTICLES) {
        // Erosion::dispatch_particle (src/erosion.cpp:132-156): droplets move
        // and erode, both thermal layers (identities skipped), smoothing with
        // the momentum fold; rain on = new droplets spawn
        if (!w->parts) return fail(HG_ERR_INVALID, "particle mode needs hg_particles_init");
        Particles& P = *w->parts;
        const Talus1 t1 = make_talus1(w);
        auto swap2 = [](float** f) { float* t = f[0]; f[0] = f[1]; f[1] = t; };
        for (int k = 0; k < nsteps; ++k) {
            PWorld cur{w->cur[S_ROCK], w->dirt[0], w->cur[S_WATER], {P.mom[0][0], P.mom[0][1], P.mom[0][2], P.mom[0][3]}};
            launch_particle_step(c, w->es, P.b, cur, (uint32_t)(w->step + 1), w->opt.rain_seed,
                                 w->opt.rain_mode != HG_RAIN_OFF, st);
            if (fused2_ok(w->n)) {  // talus passes and smoothing as fused kernels
                PWorld out{w->alt[S_ROCK], w->dirt[1], w->alt[S_WATER],
                           {P.mom[1][0], P.mom[1][1], P.mom[1][2], P.mom[1][3]}};
                float* rock_mid = reinterpret_cast<float*>(w->tc);
                int rc = launch_particle_thermal_smooth(c, t1, (float)P.count, cur, out, rock_mid, w->tma, w->err, st);
                if (rc != HG_OK) return fail(rc, "cuTensorMapEncodeTiled failed for a world buffer");
                swap(S_ROCK);
                swap(S_WATER);
                swap2(w->dirt);
                for (int ch = 0; ch < 4; ++ch) std::swap(P.mom[0][ch], P.mom[1][ch]);
                w->step += 1;
                continue;
            }
            if (c.thermal) {
                launch_thermal_out(c, w->cur[S_ROCK], w->tc, w->td, st);
                launch_thermal_in(c, w->cur[S_ROCK], w->tc, w->td, w->alt[S_ROCK], st);
                swap(S_ROCK);
            }
            if (c.Kspeed1 != 0.0f) {
                launch_thermal_out1(c, w->cur[S_ROCK], w->dirt[0], w->tc, w->td, st);
                launch_thermal_in(c, w->dirt[0], w->tc, w->td, w->dirt[1], st);
                swap2(w->dirt);
            }
            PWorld in{w->cur[S_ROCK], w->dirt[0], w->cur[S_WATER], {P.mom[0][0], P.mom[0][1], P.mom[0][2], P.mom[0][3]}};
            PWorld out{w->alt[S_ROCK], w->dirt[1], w->alt[S_WATER], {P.mom[1][0], P.mom[1][1], P.mom[1][2], P.mom[1][3]}};
            launch_particle_smooth(c, (float)P.count, in, out, st);
            swap(S_ROCK);
            swap(S_WATER);
            swap2(w->dirt);
            for (int ch = 0; ch < 4; ++ch) std::swap(P.mom[0][ch], P.mom[1][ch]);
            w->step += 1;
        }
        if (nsteps > 0) w->dev_step_valid = false;
        HG_CUDA(cudaGetLastError());
        return HG_OK;
    }
    if (mode == HG_MODE_PLAIN && w->layers == 2) {
        // the reference's two-layer step (src/erosion.cpp:158-200): thermal
        // and smoothing passes for layers whose slippage rate is 0 are
        // identities and are skipped
        auto swap2 = [](float** f) { float* t = f[0]; f[0] = f[1]; f[1] = t; };
        for (int k = 0; k < nsteps; ++k) {
            rain_pass(w, c, w->step + 1, w->cur[S_ROCK], w->dirt[0], w->cur[S_WATER], st);
            launch_flux2(c, w->cur[S_ROCK], w->dirt[0], w->cur[S_WATER], w->cur[S_FL], w->cur[S_FR], w->cur[S_FT],
                         w->cur[S_FB], w->alt[S_WATER], w->alt[S_FL], w->alt[S_FR], w->alt[S_FT], w->alt[S_FB],
                         w->u, w->v, w->vz, st);
            swap(S_WATER); swap(S_FL); swap(S_FR); swap(S_FT); swap(S_FB);
            launch_erosion2(c, w->u, w->v, w->vz, w->cur[S_ROCK], w->dirt[0], w->alt[S_ROCK], w->dirt[1],
                            w->cur[S_SED], w->sdirt[0], st);
            swap(S_ROCK);
            swap2(w->dirt);
            launch_sediment2(c, w->u, w->v, w->cur[S_SED], w->sdirt[0], w->alt[S_SED], w->sdirt[1], w->cur[S_WATER],
                             st);
            swap(S_SED);
            swap2(w->sdirt);
            if (c.thermal) {  // layer 0: drops of rock only
                launch_thermal_out(c, w->cur[S_ROCK], w->tc, w->td, st);
                launch_thermal_in(c, w->cur[S_ROCK], w->tc, w->td, w->alt[S_ROCK], st);
                swap(S_ROCK);
            }
            if (c.Kspeed1 != 0.0f) {  // layer 1: drops of rock + dirt, dirt moves
                launch_thermal_out1(c, w->cur[S_ROCK], w->dirt[0], w->tc, w->td, st);
                launch_thermal_in(c, w->dirt[0], w->tc, w->td, w->dirt[1], st);
                swap2(w->dirt);
            }
            if (c.smooth_m != 0.0f) {
                launch_smooth2(c, w->cur[S_ROCK], w->dirt[0], w->alt[S_ROCK], w->dirt[1], st);
                swap(S_ROCK);
                swap2(w->dirt);
            }
            w->step += 1;
        }
        if (nsteps > 0) w->dev_step_valid = false;
    } else if (mode == HG_MODE_PLAIN) {
        for (int k = 0; k < nsteps; ++k) {
            rain_pass(w, c, w->step + 1, w->cur[S_ROCK], nullptr, w->cur[S_WATER], st);
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
            // the dirt layer's talus pass moves nothing (its H is min(0, .) == 0);
            // smoothing changes rock when Kspeed[1] != 0
            if (c.smooth_m != 0.0f) {
                launch_smooth(c, w->cur[S_ROCK], w->alt[S_ROCK], st);
                swap(S_ROCK);
            }
            w->step += 1;
        }
        if (nsteps > 0) w->dev_step_valid = false;
    } else if (nsteps > 0 && w->layers == 2) {
        int rc = fused2_steps(w, nsteps);
        if (rc != HG_OK) return rc;
    } else if (nsteps > 0) {
        std::vector<hg_world*> one{w};
        int rc = fused_run(w->plans, one, w->tuning, w->opt.tile_y, w->opt.graph, st, w->err, nsteps);
        if (rc != HG_OK) return rc;
    }
    HG_CUDA(cudaGetLastError());
    return HG_OK;
}

int hg_set_rows(hg_world* w, int lo, int hi) {
    HG_CHECK_WORLD(w);
    if (hi < 0) hi = w->n;
    if (lo < 0 || lo > hi || hi > w->n) return fail(HG_ERR_INVALID, "rows must satisfy 0 <= lo <= hi <= n");
    w->row_lo = lo;
    w->row_hi = hi;
    return HG_OK;
}

int hg_pass(hg_world* w, int pass, int layer) {
    Range nv_range("hg_pass");
    HG_CHECK_WORLD(w);
    HG_CHECK_VALID(w);
    if (w->layers != 1) return fail(HG_ERR_UNSUPPORTED, "single passes cover one-layer worlds");
    if (pass < HG_PASS_RAIN || pass > HG_PASS_SMOOTHING) return fail(HG_ERR_INVALID, "bad pass");
    if (layer != 0 && layer != 1) return fail(HG_ERR_INVALID, "layer must be 0 or 1");
    DeviceGuard g(w->device);
    const StepConsts c = make_consts(w);
    cudaStream_t st = w->stream;
    auto swap = [&](int f) { float* t = w->cur[f]; w->cur[f] = w->alt[f]; w->alt[f] = t; };
    // the operations and buffer swaps of the one-layer per-pass step
    switch (pass) {
        case HG_PASS_RAIN:
            rain_pass(w, c, w->step + 1, w->cur[S_ROCK], nullptr, w->cur[S_WATER], st);
            break;
        case HG_PASS_FLUX:
            launch_flux(c, w->cur[S_ROCK], w->cur[S_WATER], w->cur[S_FL], w->cur[S_FR], w->cur[S_FT], w->cur[S_FB],
                        w->alt[S_WATER], w->alt[S_FL], w->alt[S_FR], w->alt[S_FT], w->alt[S_FB], w->u, w->v, w->vz,
                        st);
            swap(S_WATER); swap(S_FL); swap(S_FR); swap(S_FT); swap(S_FB);
            break;
        case HG_PASS_EROSION:
            launch_erosion(c, w->u, w->v, w->vz, w->cur[S_ROCK], w->alt[S_ROCK], w->cur[S_SED], st);
            swap(S_ROCK);
            break;
        case HG_PASS_SEDIMENT:
            launch_sediment(c, w->u, w->v, w->cur[S_SED], w->alt[S_SED], w->cur[S_WATER], st);
            swap(S_SED);
            break;
        case HG_PASS_THERMAL_FLUX:  // the empty dirt layer's talus pass moves nothing
            if (layer == 0) launch_thermal_out(c, w->cur[S_ROCK], w->tc, w->td, st);
            break;
        case HG_PASS_THERMAL_TRANSPORT:
            if (layer == 0) {
                launch_thermal_in(c, w->cur[S_ROCK], w->tc, w->td, w->alt[S_ROCK], st);
                swap(S_ROCK);
            }
            break;
        default:  // HG_PASS_SMOOTHING: the identity when Kspeed[1] == 0
            if (c.smooth_m != 0.0f) {
                launch_smooth(c, w->cur[S_ROCK], w->alt[S_ROCK], st);
                swap(S_ROCK);
            }
            break;
    }
    w->dev_step_valid = false;
    HG_CUDA(cudaGetLastError());
    return HG_OK;
}

int hg_fused_pass(hg_world* w, int which) {
    Range nv_range("hg_fused_pass");
    HG_CHECK_WORLD(w);
    HG_CHECK_VALID(w);
    if (which != 0 && which != 1) return fail(HG_ERR_INVALID, "which must be 0 (k_hydro) or 1 (k_transport)");
    if (w->layers != 1) return fail(HG_ERR_UNSUPPORTED, "fused halves cover one-layer worlds");
    const int th = 16;
    if (!fused_tile_ok(w->n, th)) return fail(HG_ERR_UNSUPPORTED, "fused mode needs n divisible by 64");
    const StepConsts c = make_consts(w);
    if (c.smooth_m != 0.0f || w->opt.rain_mode == HG_RAIN_REFERENCE)
        return fail(HG_ERR_UNSUPPORTED, "fused halves cover worlds without smoothing or the reference rain");
    if (w->row_lo % th || w->row_hi % th)
        return fail(HG_ERR_INVALID, "fused halves step whole tile rows: the row range must be multiples of 16");
    DeviceGuard g(w->device);
    cudaStream_t st = w->stream;
    if (!w->dev_step_valid) {
        k_set_u64<<<1, 1, 0, st>>>(w->d_step, (unsigned long long)w->step);
        w->dev_step_valid = true;
    }
    TerrainSrc src{};
    src.c = c;
    src.rain = make_rain_base(w);
    src.step = w->d_step;
    for (int f = 0; f < S_COUNT; ++f) {
        src.in[f] = w->cur[f];
        src.out[f] = w->alt[f];
    }
    src.u = w->u;
    src.v = w->v;
    src.s_ero = w->s_ero;
    src.b_ero = w->b_ero;
    TerrainDesc td;
    if (!fill_desc(td, src, th, 0, w->tma)) return fail(HG_ERR_CUDA, "cuTensorMapEncodeTiled failed for a world buffer");
    const int tiles_x = w->n / 64;
    launch_fused_half(td, th, which, (w->row_lo / th) * tiles_x, ((w->row_hi - w->row_lo) / th) * tiles_x, w->err,
                      st);
    if (which == 1) {  // the step's outputs become the state (k_transport advanced the device counter)
        for (int f = 0; f < S_COUNT; ++f) std::swap(w->cur[f], w->alt[f]);
        w->step += 1;
    }
    HG_CUDA(cudaGetLastError());
    return HG_OK;
}

int hg_world_rows(hg_world* w, int field, int y0, int y1, float* host, int write) {
    HG_CHECK_WORLD(w);
    if (!host) return fail(HG_ERR_INVALID, "null host pointer");
    if (y0 < 0 || y0 > y1 || y1 > w->n) return fail(HG_ERR_INVALID, "rows must satisfy 0 <= y0 <= y1 <= n");
    float* d = nullptr;
    size_t per_cell = 1;
    if (field == HG_ROWS_THERMAL_C || field == HG_ROWS_THERMAL_D) {
        d = reinterpret_cast<float*>(field == HG_ROWS_THERMAL_C ? w->tc : w->td);
        per_cell = 4;
    } else if (field == HG_ROWS_ERODED_ROCK || field == HG_ROWS_ERODED_SEDIMENT) {
        d = field == HG_ROWS_ERODED_ROCK ? w->b_ero : w->s_ero;
    } else {
        d = field_ptr(w, field);
    }
    if (!d) return fail(HG_ERR_INVALID, "bad field id");
    DeviceGuard g(w->device);
    const size_t off = (size_t)y0 * w->n * per_cell, count = (size_t)(y1 - y0) * w->n * per_cell;
    if (count) {
        if (write)
            HG_CUDA(cudaMemcpyAsync(d + off, host, count * sizeof(float), cudaMemcpyHostToDevice, w->stream));
        else
            HG_CUDA(cudaMemcpyAsync(host, d + off, count * sizeof(float), cudaMemcpyDeviceToHost, w->stream));
    }
    HG_CUDA(cudaStreamSynchronize(w->stream));
    return HG_OK;
}

int hg_world_tuning(const hg_world* w, int* tile_y, int* graph, double ms[4]) {
    HG_CHECK_WORLD(w);
    if (tile_y) *tile_y = w->tuning.th;
    if (graph) *graph = w->tuning.graph;
    if (ms)
        for (int k = 0; k < 4; ++k) ms[k] = w->tuning.ms[k];
    return HG_OK;
}

// ---- batches ---------------------------------------------------------------------

int hg_batch_create(hg_world* const* worlds, int count, hg_batch** out) {
    if (!out) return fail(HG_ERR_INVALID, "null output pointer");
    *out = nullptr;
    if (!worlds || count < 1) return fail(HG_ERR_INVALID, "a batch needs at least one world");
    if (count > MAX_BATCH) return fail(HG_ERR_UNSUPPORTED, "a batch holds at most 128 worlds");
    for (int i = 0; i < count; ++i) {
        if (!worlds[i]) return fail(HG_ERR_INVALID, "null world in batch");
        if (worlds[i]->device != worlds[0]->device) return fail(HG_ERR_INVALID, "batch worlds must share a device");
        for (int j = 0; j < i; ++j)
            if (worlds[j] == worlds[i]) return fail(HG_ERR_INVALID, "a world appears twice in the batch");
    }
    DeviceGuard g(worlds[0]->device);
    hg_batch* b = new (std::nothrow) hg_batch();
    if (!b) return fail(HG_ERR_OOM, "host allocation failed");
    b->worlds.assign(worlds, worlds + count);
    b->device = worlds[0]->device;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(b->err, 0, sizeof(int));
    if (e != cudaSuccess) {
        if (b->stream) cudaStreamDestroy(b->stream);
        if (b->ev) cudaEventDestroy(b->ev);
        cudaFree(b->err);
        delete b;
        return cuda_fail(e, "batch creation");
    }
    *out = b;
    return HG_OK;
}

int hg_batch_destroy(hg_batch* b) {
    if (!b) return HG_OK;
    DeviceGuard g(b->device);
    cudaStreamSynchronize(b->stream);
    for (Plan*& p : b->plans) destroy_plan(p);
    cudaEventDestroy(b->ev);
    cudaStreamDestroy(b->stream);
    cudaFree(b->err);
    delete b;
    return HG_OK;
}

int hg_batch_step(hg_batch* b, int nsteps, int mode) {
    Range nv_range("hg_batch_step");
    if (!b) return fail(HG_ERR_INVALID, "null batch");
    if (nsteps < 0) return fail(HG_ERR_INVALID, "nsteps must be >= 0");
    if (mode != HG_MODE_PLAIN && mode != HG_MODE_FUSED && mode != HG_MODE_FUSED_PER_WORLD)
        return fail(HG_ERR_INVALID, "bad mode");
    if (nsteps == 0) return HG_OK;
    for (hg_world* w : b->worlds) {
        HG_CHECK_VALID(w);
        if (rows_restricted(w)) return fail(HG_ERR_UNSUPPORTED, "a batch steps whole worlds (hg_set_rows is set)");
    }
    DeviceGuard g(b->device);
    bool two_layer = false;  // the table launch covers one-layer worlds
    for (hg_world* w : b->worlds) two_layer = two_layer || w->layers == 2;
    if (mode != HG_MODE_FUSED || two_layer) {  // every world on its own stream, its own launches
        for (hg_world* w : b->worlds) {
            int rc = hg_step(w, nsteps, mode == HG_MODE_PLAIN ? HG_MODE_PLAIN : HG_MODE_FUSED);
            if (rc != HG_OK) return rc;
        }
        return HG_OK;
    }
    const hg_step_options& o = b->worlds[0]->opt;
    const bool autotune = o.tile_y == HG_AUTO && o.graph == HG_AUTO;
    auto join_worlds = [&]() -> int {  // batch stream after every world's stream
        for (hg_world* w : b->worlds) {
            HG_CUDA(cudaEventRecord(b->ev, w->stream));
            HG_CUDA(cudaStreamWaitEvent(b->stream, b->ev, 0));
        }
        return HG_OK;
    };
    auto release_worlds = [&]() -> int {  // every world's stream after the batch stream
        HG_CUDA(cudaEventRecord(b->ev, b->stream));
        for (hg_world* w : b->worlds) HG_CUDA(cudaStreamWaitEvent(w->stream, b->ev, 0));
        return HG_OK;
    };
    auto per_world = [&](int k) -> int {
        for (hg_world* w : b->worlds) {
            int rc = hg_step(w, k, HG_MODE_FUSED);
            if (rc != HG_OK) return rc;
        }
        return HG_OK;
    };
    if (autotune && b->tuning.th == 0 && nsteps >= 12) {
        // Two untimed steps of per-world launches build (and capture) the
        // worlds' own plans; the next two are timed.  fused_run then times the
        // table variants; the faster form serves every later call.
        cudaEvent_t e0, e1;
        HG_CUDA(cudaEventCreate(&e0));
        HG_CUDA(cudaEventCreate(&e1));
        int rc = per_world(2);
        if (rc == HG_OK) rc = join_worlds();
        if (rc == HG_OK) rc = cudaEventRecord(e0, b->stream) == cudaSuccess ? release_worlds() : HG_ERR_CUDA;
        if (rc == HG_OK) rc = per_world(2);
        if (rc == HG_OK) rc = join_worlds();
        if (rc == HG_OK && cudaEventRecord(e1, b->stream) != cudaSuccess) rc = HG_ERR_CUDA;
        if (rc == HG_OK && cudaEventSynchronize(e1) != cudaSuccess) rc = HG_ERR_CUDA;
        float ms = 0;
        if (rc == HG_OK) cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc != HG_OK) return rc == HG_ERR_CUDA ? cuda_fail(cudaGetLastError(), "batch tuning") : rc;
        b->tuning.ms_per_world = ms / 2.0;
        nsteps -= 4;
        if ((rc = join_worlds()) != HG_OK) return rc;
        rc = fused_run(b->plans, b->worlds, b->tuning, o.tile_y, o.graph, b->stream, b->err, 8);
        if (rc != HG_OK) return rc;
        nsteps -= 8;
        double best = 1e30;
        for (double m : b->tuning.ms) best = std::min(best, m);
        b->tuning.per_world = b->tuning.ms_per_world < best ? 1 : 0;
        char m[120];
        std::snprintf(m, sizeof m, "autotuner: batch of %zu worlds, %s (%.4f ms/step per world's launches)",
                      b->worlds.size(), b->tuning.per_world ? "per-world launches" : "one table launch",
                      b->tuning.ms_per_world);
        log_msg(HG_LOG_INFO, m);
        if ((rc = release_worlds()) != HG_OK) return rc;
    }
    if (autotune && b->tuning.per_world) return per_world(nsteps);
    // one table launch per kernel for every world: ordered after the worlds' streams
    int rc = join_worlds();
    if (rc != HG_OK) return rc;
    rc = fused_run(b->plans, b->worlds, b->tuning, o.tile_y, o.graph, b->stream, b->err, nsteps);
    int rc2 = release_worlds();
    return rc != HG_OK ? rc : rc2;
}

int hg_batch_sync(hg_batch* b) {
    if (!b) return fail(HG_ERR_INVALID, "null batch");
    DeviceGuard g(b->device);
    HG_CUDA(cudaStreamSynchronize(b->stream));
    int flag = 0;
    HG_CUDA(cudaMemcpy(&flag, b->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) {
        HG_CUDA(cudaMemset(b->err, 0, sizeof(int)));
        for (hg_world* w : b->worlds) w->invalid = true;
        return fail(HG_ERR_TIMEOUT, "a fused-step tile load did not arrive within its bounded wait; "
                                    "the batch's fields are undefined until its worlds are re-initialised or loaded");
    }
    for (hg_world* w : b->worlds) {
        int rc = hg_sync(w);
        if (rc != HG_OK) return rc;
    }
    return HG_OK;
}

int hg_batch_stream(const hg_batch* b, void** stream) {
    if (!b || !stream) return fail(HG_ERR_INVALID, "null argument");
    *stream = (void*)b->stream;
    return HG_OK;
}

int hg_batch_tuning(const hg_batch* b, int* tile_y, int* graph, double ms[4]) {
    if (!b) return fail(HG_ERR_INVALID, "null batch");
    if (tile_y) *tile_y = b->tuning.th;
    if (graph) *graph = b->tuning.graph;
    if (ms)
        for (int k = 0; k < 4; ++k) ms[k] = b->tuning.ms[k];
    return HG_OK;
}

int hg_batch_launch_form(const hg_batch* b, int* per_world, double* ms_per_world) {
    if (!b) return fail(HG_ERR_INVALID, "null batch");
    if (per_world) *per_world = b->tuning.per_world;
    if (ms_per_world) *ms_per_world = b->tuning.ms_per_world;
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
        w->invalid = true;
        return fail(HG_ERR_TIMEOUT, "a fused-step tile load did not arrive within its bounded wait; "
                                    "the world's fields are undefined until it is re-initialised or loaded");
    }
    return HG_OK;
}

// ---- differentiation ---------------------------------------------------------------

struct hg_tape {
    hg_world* w = nullptr;
    int nsteps = 0, K = 0, nseg = 0;
    uint64_t step0 = 0;
    bool recorded = false;
    bool last_ready = false;  // the last segment's states and intermediates are in seg / slots
    float* ckpt = nullptr;   // nseg states: the input of each segment's first step
    int nbuf = 1;            // segment buffers: 2 lets the next segment's recompute overlap a reverse sweep
    float* seg = nullptr;    // nbuf x K states: slot j >= 1 the input of a segment's step j,
                             // slot 0 receives the (unused) output of its last step
    float* slots = nullptr;  // nbuf x K x (u, v, eroded sediment, eroded rock) of a segment's steps
    float* adj = nullptr;    // 2 adjoint states (own terms), alternating A / R
    float* pk = nullptr;     // their 2 x ADJ_PACKET_FIELDS neighbour packets
    float* aux = nullptr;    // 2 sediment-adjoint buffers, du, dv, rock adjoints for the talus reverse
    float* dks = nullptr;    // per-cell Ks gradient
    unsigned long long* d_step = nullptr;  // step counter of the recompute launches
    cudaStream_t rstream = nullptr;        // recompute stream (nbuf == 2)
    cudaEvent_t ev_rec[2] = {}, ev_rev[2] = {};  // per buffer: recompute done, reverse sweep done
    TmaCache tma;
};

namespace {
constexpr int kStateFields = 7;
constexpr int kSlotFields = 4;  // u, v, eroded sediment, eroded rock
constexpr int kAuxFields = 5;   // 2 sediment-adjoint buffers, du, dv, eroded-rock adjoint

AdjFields fields_at(float* base, size_t c) {
    AdjFields f;
    f.b = base;
    f.d = base + c;
    f.s = base + 2 * c;
    for (int k = 0; k < 4; ++k) f.f[k] = base + (3 + k) * c;
    return f;
}

void free_tape(hg_tape* t) {
    cudaFree(t->ckpt); cudaFree(t->seg); cudaFree(t->slots); cudaFree(t->adj); cudaFree(t->pk);
    cudaFree(t->aux); cudaFree(t->dks); cudaFree(t->d_step);
    for (int b = 0; b < 2; ++b) {
        if (t->ev_rec[b]) cudaEventDestroy(t->ev_rec[b]);
        if (t->ev_rev[b]) cudaEventDestroy(t->ev_rev[b]);
    }
    if (t->rstream) cudaStreamDestroy(t->rstream);
}

}  // namespace

// A world that is destroyed before its tapes frees their device memory and
// leaves each tape a husk: hg_tape_destroy then only deletes the handle, and
// the tape's other entry points report HG_ERR_STATE.
extern "C++" void hg::release_tapes(hg_world* w) {
    for (hg_tape* t : w->tapes) {
        free_tape(t);
        t->w = nullptr;
    }
    w->tapes.clear();
}

namespace {

// state fields of a world (current buffers) -> contiguous state at dst
int copy_state_out(hg_world* w, float* dst, cudaStream_t st) {
    size_t c = cells(w);
    for (int f = 0; f < kStateFields; ++f)
        HG_CUDA(cudaMemcpyAsync(dst + f * c, w->cur[f], c * sizeof(float), cudaMemcpyDeviceToDevice, st));
    return HG_OK;
}

size_t tape_bytes(size_t c, int nsteps, int K, int nbuf) {
    const size_t nseg = (size_t)(nsteps + K - 1) / K;
    return (nseg * kStateFields + (size_t)nbuf * K * (kStateFields + kSlotFields) + 2 * kStateFields +
            2 * ADJ_PACKET_FIELDS + kAuxFields + 1) * c * sizeof(float);
}
}  // namespace

int hg_tape_create(hg_world* w, int nsteps, int ckpt_every, hg_tape** out) {
    HG_CHECK_WORLD(w);
    if (!out) return fail(HG_ERR_INVALID, "null output pointer");
    *out = nullptr;
    if (nsteps < 1) return fail(HG_ERR_INVALID, "nsteps must be >= 1");
    if (!adjoint_covers(w)) return fail(HG_ERR_UNSUPPORTED, "the adjoint covers one-layer worlds without smoothing (Kspeed[1] == 0) or the reference rain");
    if (!fused_tile_ok(w->n, 16) || !adjoint_tile_ok(w->n))
        return fail(HG_ERR_UNSUPPORTED, "the adjoint needs n divisible by 64");
    DeviceGuard g(w->device);
    const size_t c = cells(w);
    // Checkpoints (nsteps/K states) plus segment buffers (K states and
    // slots each), within the free memory less a reserve (a tenth of it, at
    // least 4 GiB, for the caller's later allocations).  The backward
    // recomputes every segment but the last once, nsteps - K steps in all,
    // so HG_AUTO takes the longest interval that fits (K = nsteps: nothing
    // is recomputed); tape memory is smallest near K = sqrt(7 nsteps / 11),
    // the fallback when nothing fits.  A second segment buffer, when it
    // fits too, lets the recompute overlap the reverse sweep.
    size_t free_b = 0, total_b = 0;
    size_t budget = (size_t)-1;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
        const size_t reserve = std::max<size_t>(free_b / 10, (size_t)4 << 30);
        budget = free_b > reserve ? free_b - reserve : 0;
    }
    int K = ckpt_every, nbuf = 1;
    if (K == HG_AUTO || K <= 0) {
        K = 0;
        for (int cand = nsteps; cand >= 1 && K == 0; --cand)
            if (tape_bytes(c, nsteps, cand, 1) <= budget) K = cand;
        if (K == 0)  // nothing fits: let the allocation report it
            K = std::min(nsteps, std::max(1, (int)std::lround(std::sqrt(7.0 * nsteps / 11.0))));
        nbuf = K < nsteps && tape_bytes(c, nsteps, K, 2) <= budget ? 2 : 1;
    } else {
        K = std::min(K, nsteps);
        nbuf = tape_bytes(c, nsteps, K, 2) <= budget ? 2 : 1;
    }
    hg_tape* t = new (std::nothrow) hg_tape();
    if (!t) return fail(HG_ERR_OOM, "host allocation failed");
    t->w = w;
    t->nsteps = nsteps;
    t->K = K;
    t->nseg = (nsteps + K - 1) / K;
    t->nbuf = t->nseg > 1 ? nbuf : 1;
    const size_t fb = c * sizeof(float);
    cudaError_t e = cudaMalloc((void**)&t->ckpt, (size_t)t->nseg * kStateFields * fb);
    if (e == cudaSuccess) e = cudaMalloc((void**)&t->seg, (size_t)t->nbuf * K * kStateFields * fb);
    if (e == cudaSuccess) e = cudaMalloc((void**)&t->slots, (size_t)t->nbuf * K * kSlotFields * fb);
    if (e == cudaSuccess && t->nbuf == 2) {
        e = cudaStreamCreateWithFlags(&t->rstream, cudaStreamNonBlocking);
        for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
            e = cudaEventCreateWithFlags(&t->ev_rec[b], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&t->ev_rev[b], cudaEventDisableTiming);
        }
    }
    if (e == cudaSuccess) e = cudaMalloc((void**)&t->adj, 2 * kStateFields * fb);
    if (e == cudaSuccess) e = cudaMalloc((void**)&t->pk, 2 * ADJ_PACKET_FIELDS * fb);
    if (e == cudaSuccess) e = cudaMalloc((void**)&t->aux, kAuxFields * fb);
    if (e == cudaSuccess) e = cudaMalloc((void**)&t->dks, fb);
    if (e == cudaSuccess) e = cudaMalloc((void**)&t->d_step, sizeof(unsigned long long));
    if (e != cudaSuccess) {
        free_tape(t);
        delete t;
        int code = e == cudaErrorMemoryAllocation ? HG_ERR_OOM : HG_ERR_CUDA;
        cudaGetLastError();
        return fail(code, std::string("tape allocation: ") + cudaGetErrorString(e));
    }
    w->tapes.push_back(t);
    *out = t;
    return HG_OK;
}

int hg_tape_destroy(hg_tape* t) {
    if (!t) return HG_OK;
    if (t->w) {  // else its world's destruction released the buffers already
        DeviceGuard g(t->w->device);
        cudaStreamSynchronize(t->w->stream);
        auto& v = t->w->tapes;
        v.erase(std::remove(v.begin(), v.end(), t), v.end());
        free_tape(t);
    }
    delete t;
    return HG_OK;
}

int hg_tape_info(const hg_tape* t, int* nsteps, int* ckpt_every) {
    if (!t) return fail(HG_ERR_INVALID, "null tape");
    if (!t->w) return fail(HG_ERR_STATE, "the tape's world was destroyed");
    if (nsteps) *nsteps = t->nsteps;
    if (ckpt_every) *ckpt_every = t->K;
    return HG_OK;
}

// Segments: the first holds the remainder, nsteps - (nseg - 1) K steps (1 to
// K), every later one K steps, so the last segment, which the forward leaves
// in the segment buffers, is a whole interval and the backward recomputes
// nsteps - K steps.
int seg_len(const hg_tape* t, int s) { return s == 0 ? t->nsteps - (t->nseg - 1) * t->K : t->K; }
// Steps before segment s (relative to the tape's first step).
uint64_t seg_start(const hg_tape* t, int s) { return s == 0 ? 0 : (uint64_t)seg_len(t, 0) + (uint64_t)(s - 1) * t->K; }

// Segment buffer b: its K states and K slot groups.
float* seg_buf(hg_tape* t, int b) { return t->seg + (size_t)b * t->K * kStateFields * cells(t->w); }
float* slot_buf(hg_tape* t, int b) { return t->slots + (size_t)b * t->K * kSlotFields * cells(t->w); }

// Recomputes segment s from its checkpoint with the fused step on stream
// `st` into segment buffer b: step j reads its input state (checkpoint or
// state slot j) and writes the next state into state slot j + 1 and u, v,
// eroded sediment and eroded rock into its slot group; the last step's state
// goes to `last_out` (7 fields) or state slot 0.  No state copies.
int recompute_segment(hg_tape* t, int s, int len, const StepConsts& cst, int th, float* const* last_out, int b,
                      cudaStream_t st) {
    hg_world* w = t->w;
    const size_t c = cells(w), sf = kStateFields * c;
    float* segb = seg_buf(t, b);
    float* slotb = slot_buf(t, b);
    k_set_u64<<<1, 1, 0, st>>>(t->d_step, (unsigned long long)(t->step0 + seg_start(t, s)));
    TerrainSrc src{};
    src.c = cst;
    src.rain = make_rain_base(w);
    src.step = t->d_step;
    TerrainDesc td;
    for (int j = 0; j < len; ++j) {
        const float* in = j == 0 ? t->ckpt + (size_t)s * sf : segb + (size_t)j * sf;
        float* outp = segb + (size_t)(j + 1 < len ? j + 1 : 0) * sf;
        for (int f = 0; f < S_COUNT; ++f) {
            src.in[f] = in + f * c;
            src.out[f] = (j + 1 == len && last_out) ? last_out[f] : outp + f * c;
        }
        float* sl = slotb + (size_t)j * kSlotFields * c;
        src.u = sl;
        src.v = sl + c;
        src.s_ero = sl + 2 * c;
        src.b_ero = sl + 3 * c;
        if (!fill_desc(td, src, th, 0, t->tma))
            return fail(HG_ERR_CUDA, "cuTensorMapEncodeTiled failed for a tape buffer");
        launch_fused_one(td, th, w->err, st);
    }
    HG_CUDA(cudaGetLastError());
    return HG_OK;
}

int hg_forward(hg_tape* t) {
    Range nv_range("hg_forward");
    if (!t) return fail(HG_ERR_INVALID, "null tape");
    if (!t->w) return fail(HG_ERR_STATE, "the tape's world was destroyed");
    hg_world* w = t->w;
    HG_CHECK_VALID(w);
    if (!adjoint_covers(w)) return fail(HG_ERR_UNSUPPORTED, "the adjoint covers one-layer worlds without smoothing (Kspeed[1] == 0) or the reference rain");
    if (rows_restricted(w)) return fail(HG_ERR_UNSUPPORTED, "a tape steps the whole world (hg_set_rows is set)");
    DeviceGuard g(w->device);
    t->step0 = w->step;
    const size_t c = cells(w);
    for (int s = 0; s < t->nseg; ++s) {
        int rc = copy_state_out(w, t->ckpt + (size_t)s * kStateFields * c, w->stream);
        if (rc != HG_OK) return rc;
        const int len = seg_len(t, s);
        if (s + 1 < t->nseg) {
            rc = hg_step(w, len, HG_MODE_FUSED);
            if (rc != HG_OK) return rc;
            continue;
        }
        // the last segment steps through the tape's buffers: its states and
        // intermediates stay for the backward sweep, the final state lands in
        // the world's alternate buffers
        rc = recompute_segment(t, s, len, make_consts(w), w->tuning.th ? w->tuning.th : 16, w->alt, 0, w->stream);
        if (rc != HG_OK) return rc;
        for (int f = 0; f < S_COUNT; ++f) std::swap(w->cur[f], w->alt[f]);
        w->step += (uint64_t)len;
        w->dev_step_valid = false;
        const float* sl = slot_buf(t, 0) + (size_t)(len - 1) * kSlotFields * c;
        HG_CUDA(cudaMemcpyAsync(w->u, sl, c * sizeof(float), cudaMemcpyDeviceToDevice, w->stream));
        HG_CUDA(cudaMemcpyAsync(w->v, sl + c, c * sizeof(float), cudaMemcpyDeviceToDevice, w->stream));
    }
    t->recorded = true;
    t->last_ready = true;
    return HG_OK;
}

int hg_backward(hg_tape* t, const float* dL_drock_final, float* dL_dks, float* dL_drock0) {
    Range nv_range("hg_backward");
    if (!t) return fail(HG_ERR_INVALID, "null tape");
    if (!t->w) return fail(HG_ERR_STATE, "the tape's world was destroyed");
    if (!t->recorded) return fail(HG_ERR_STATE, "hg_forward has not recorded this tape");
    if (!dL_drock_final) return fail(HG_ERR_INVALID, "null final-rock adjoint");
    hg_world* w = t->w;
    if (!adjoint_covers(w)) return fail(HG_ERR_UNSUPPORTED, "the adjoint covers one-layer worlds without smoothing (Kspeed[1] == 0) or the reference rain");
    DeviceGuard g(w->device);
    cudaStream_t st = w->stream;
    const size_t c = cells(w), sf = kStateFields * c;
    const StepConsts cst = make_consts(w);
    const int th = w->tuning.th ? w->tuning.th : 16;
    // state adjoints alternate between two buffers of own terms and packets
    AdjFields own[2] = {fields_at(t->adj, c), fields_at(t->adj + sf, c)};
    float* pkb[2] = {t->pk, t->pk + ADJ_PACKET_FIELDS * c};
    auto view = [&](int k) {
        AdjView v;
        v.b = own[k].b;
        v.d = own[k].d;
        for (int d = 0; d < 4; ++d) {
            v.f[d] = own[k].f[d];
            v.pdh[d] = pkb[k] + (size_t)d * c;
            v.pin[d] = pkb[k] + (size_t)(4 + d) * c;
        }
        v.pdx = pkb[k] + 8 * c;
        v.pdz = pkb[k] + 9 * c;
        return v;
    };
    float* dse[2] = {t->aux, t->aux + c};
    float* du = t->aux + 2 * c;
    float* dv = t->aux + 3 * c;
    float* gbe = t->aux + 4 * c;  // adjoint of the eroded rock
    // the final state's adjoint: rock only, no packets
    HG_CUDA(cudaMemsetAsync(t->adj, 0, 2 * sf * sizeof(float), st));
    HG_CUDA(cudaMemsetAsync(t->pk, 0, 2 * ADJ_PACKET_FIELDS * c * sizeof(float), st));
    HG_CUDA(cudaMemsetAsync(t->aux, 0, 2 * c * sizeof(float), st));  // scatter targets start at zero
    HG_CUDA(cudaMemcpyAsync(own[0].b, dL_drock_final, c * sizeof(float), cudaMemcpyDeviceToDevice, st));
    HG_CUDA(cudaMemsetAsync(t->dks, 0, c * sizeof(float), st));
    // segment s lives in buffer (nseg - 1 - s) % nbuf; with two buffers the
    // next segment's recompute runs on the recompute stream while this
    // segment's reverse sweep runs on the world's stream
    const bool overlap = t->nbuf == 2;
    auto buf_of = [&](int s) { return overlap ? (t->nseg - 1 - s) & 1 : 0; };
    int bcur = 0;
    auto slot_of = [&](int j) {
        const float* sl = slot_buf(t, bcur) + (size_t)j * kSlotFields * c;
        return AdjSlot{sl, sl + c, sl + 2 * c};
    };
    auto recompute = [&](int s, cudaStream_t rs) -> int {
        const int b = buf_of(s);
        if (overlap) HG_CUDA(cudaStreamWaitEvent(rs, t->ev_rev[b], 0));  // the sweep that used b is done
        int rc = recompute_segment(t, s, seg_len(t, s), cst, th, nullptr, b, rs);
        if (rc != HG_OK) return rc;
        if (overlap) HG_CUDA(cudaEventRecord(t->ev_rec[b], rs));
        return HG_OK;
    };
    if (overlap) {
        // the recompute stream starts after everything queued on the world's stream
        HG_CUDA(cudaEventRecord(t->ev_rev[0], st));
        HG_CUDA(cudaEventRecord(t->ev_rev[1], st));
    }
    if (!t->last_ready) {  // the forward left the last segment in buffer 0 otherwise
        int rc = recompute(t->nseg - 1, overlap ? t->rstream : st);
        if (rc != HG_OK) return rc;
    }
    AdjCellArgs args;
    args.c = cst;
    args.du = du;
    args.dv = dv;
    args.dks = t->dks;
    int cur = 0;      // buffer holding the adjoint of the next reversed step's output
    uint64_t m = 0;   // reversed steps so far: step m uses dse[m & 1]
    for (int s = t->nseg - 1; s >= 0; --s) {
        const int len = seg_len(t, s);
        bcur = buf_of(s);
        if (overlap) {
            HG_CUDA(cudaStreamWaitEvent(st, t->ev_rec[bcur], 0));
            if (s > 0) {  // the previous segment into the other buffer, concurrently
                int rc = recompute(s - 1, t->rstream);
                if (rc != HG_OK) return rc;
            }
        } else if (s + 1 < t->nseg) {
            int rc = recompute(s, st);
            if (rc != HG_OK) return rc;
        }
        // the segment's last step: its sediment pass reversed on its own
        launch_adjoint_sediment(cst, slot_of(len - 1), own[cur].s, dse[m & 1], du, dv, st);
        for (int j = len - 1; j >= 0; --j, ++m) {
            const float* xin = j == 0 ? t->ckpt + (size_t)s * sf : seg_buf(t, bcur) + (size_t)j * sf;
            for (int f = 0; f < kStateFields; ++f)
                if (!t->tma.get(xin + f * c, w->n, adjoint_box_rows(), &args.maps[f]))
                    return fail(HG_ERR_CUDA, "cuTensorMapEncodeTiled failed for a tape buffer");
            args.rain = make_rain(w, t->step0 + seg_start(t, s) + j + 1);
            args.A = view(cur);
            args.dse = dse[m & 1];
            args.dse_prev = dse[(m + 1) & 1];
            args.gbe = nullptr;
            if (cst.thermal) {  // reverse the talus passes first: A's rock -> eroded rock's adjoint
                CUtensorMap mb;
                const float* be = slot_of(j).u + 3 * c;
                if (!t->tma.get(be, w->n, adjoint_thermal_box_rows(), &mb))
                    return fail(HG_ERR_CUDA, "cuTensorMapEncodeTiled failed for a tape buffer");
                launch_adjoint_thermal(cst, mb, view(cur), gbe, w->err, st);
                args.gbe = gbe;
            }
            args.scatter_prev = j > 0 ? 1 : 0;
            args.prev = j > 0 ? slot_of(j - 1) : AdjSlot{nullptr, nullptr, nullptr};
            const AdjFields& R = own[cur ^ 1];
            args.rb = R.b;
            args.rd = R.d;
            args.rs = R.s;
            AdjView rv = view(cur ^ 1);
            for (int d = 0; d < 4; ++d) {
                args.rf[d] = R.f[d];
                args.pdh[d] = const_cast<float*>(rv.pdh[d]);
                args.pin[d] = const_cast<float*>(rv.pin[d]);
            }
            args.pdx = const_cast<float*>(rv.pdx);
            args.pdz = const_cast<float*>(rv.pdz);
            launch_adjoint_cell(args, w->err, st);
            cur ^= 1;
        }
        if (overlap) HG_CUDA(cudaEventRecord(t->ev_rev[bcur], st));
    }
    if (t->nseg > t->nbuf) t->last_ready = false;  // other segments' recomputes reused buffer 0
    if (dL_drock0) launch_adjoint_final(w->n, view(cur), dL_drock0, st);
    if (dL_dks) HG_CUDA(cudaMemcpyAsync(dL_dks, t->dks, c * sizeof(float), cudaMemcpyDeviceToDevice, st));
    HG_CUDA(cudaGetLastError());
    return HG_OK;
}

int hg_mse(hg_world* w, const float* target, double* loss, float* dL_drock) {
    HG_CHECK_WORLD(w);
    if (!target || !loss) return fail(HG_ERR_INVALID, "null target or loss");
    DeviceGuard g(w->device);
    const int parts = reduction_parts();
    double* res = w->red_d + 8 * parts;
    launch_mse(w->cur[S_ROCK], target, cells(w), dL_drock, w->red_d, parts, res, w->stream);
    HG_CUDA(cudaGetLastError());
    HG_CUDA(cudaMemcpyAsync(loss, res, sizeof(double), cudaMemcpyDeviceToHost, w->stream));
    HG_CUDA(cudaStreamSynchronize(w->stream));
    return HG_OK;
}

int hg_default_fit_settings(hg_fit_settings* out) {
    if (!out) return fail(HG_ERR_INVALID, "null output");
    out->nsteps = 256;
    out->ckpt_every = 32;
    out->iters = 8;
    out->ks_step = 0.01f;
    out->ks_min = 0.005f;
    out->ks_max = 0.5f;
    out->rock_step = 0.0f;
    return HG_OK;
}

namespace {
// device scratch of one fit: the loss adjoint, the two gradients and the losses
struct FitScratch {
    float* g = nullptr;
    float* dks = nullptr;
    float* db0 = nullptr;
    double* losses = nullptr;
    hg_tape* tape = nullptr;
    ~FitScratch() {
        cudaFree(g); cudaFree(dks); cudaFree(db0); cudaFree(losses);
        if (tape) hg_tape_destroy(tape);
    }
};
}  // namespace

int hg_inverse_fit(hg_world* w, const float* target, float* ks, float* rock0, const hg_fit_settings* s,
                   double* losses, double* grad_norms) {
    Range nv_range("hg_inverse_fit");
    HG_CHECK_WORLD(w);
    if (!s) return fail(HG_ERR_INVALID, "null fit settings");
    if (!target || !rock0 || !losses) return fail(HG_ERR_INVALID, "null target, initial rock or losses");
    HG_CHECK_VALID(w);
    if (s->iters < 1) return fail(HG_ERR_INVALID, "iters must be >= 1");
    if (!(s->ks_step >= 0.0f) || !(s->rock_step >= 0.0f)) return fail(HG_ERR_INVALID, "steps must be >= 0");
    if (s->ks_step > 0.0f && !ks) return fail(HG_ERR_INVALID, "fitting Ks needs a Ks buffer");
    if (ks && !(s->ks_min >= 0.0f && s->ks_min <= s->ks_max))
        return fail(HG_ERR_INVALID, "need 0 <= ks_min <= ks_max");
    DeviceGuard g(w->device);
    cudaStream_t st = w->stream;
    const size_t c = cells(w), fb = c * sizeof(float);
    FitScratch f;
    int rc = hg_tape_create(w, s->nsteps, s->ckpt_every, &f.tape);
    if (rc != HG_OK) return rc;
    cudaError_t e = cudaMalloc((void**)&f.g, fb);
    if (e == cudaSuccess && s->ks_step > 0.0f) e = cudaMalloc((void**)&f.dks, fb);
    if (e == cudaSuccess && s->rock_step > 0.0f) e = cudaMalloc((void**)&f.db0, fb);
    if (e == cudaSuccess) e = cudaMalloc((void**)&f.losses, sizeof(double) * 2 * (size_t)s->iters);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(HG_ERR_OOM, "device allocation failed for the fit's gradients");
    }
    if (ks) {
        HG_CUDA(cudaMemcpyAsync(w->ks, ks, fb, cudaMemcpyDeviceToDevice, st));
        if (!w->ks_on) {
            w->ks_on = true;
            w->version += 1;
        }
    }
    const uint64_t step0 = w->step;
    const int parts = reduction_parts();
    for (int it = 0; it < s->iters; ++it) {
        rc = zero_state(w);
        if (rc != HG_OK) return rc;
        HG_CUDA(cudaMemcpyAsync(w->cur[S_ROCK], rock0, fb, cudaMemcpyDeviceToDevice, st));
        w->step = step0;
        w->dev_step_valid = false;
        rc = hg_forward(f.tape);
        if (rc != HG_OK) return rc;
        launch_mse(w->cur[S_ROCK], target, c, f.g, w->red_d, parts, f.losses + it, st);
        rc = hg_backward(f.tape, f.g, f.dks, f.db0);
        if (rc != HG_OK) return rc;
        if (grad_norms) {  // squared norm over the fitted fields, FP64
            double* sq = f.losses + s->iters + it;
            HG_CUDA(cudaMemsetAsync(sq, 0, sizeof(double), st));
            if (f.dks) launch_add_sumsq(f.dks, c, w->red_d, parts, sq, st);
            if (f.db0) launch_add_sumsq(f.db0, c, w->red_d, parts, sq, st);
        }
        // the Ks field is read by the next forward only, after both gradients exist
        if (s->ks_step > 0.0f) launch_descend(w->ks, f.dks, c, s->ks_step, s->ks_min, s->ks_max, w->red_f, parts, st);
        if (s->rock_step > 0.0f)
            launch_descend(rock0, f.db0, c, s->rock_step, -FLT_MAX, FLT_MAX, w->red_f, parts, st);
        HG_CUDA(cudaGetLastError());
    }
    if (ks) HG_CUDA(cudaMemcpyAsync(ks, w->ks, fb, cudaMemcpyDeviceToDevice, st));
    HG_CUDA(cudaMemcpyAsync(losses, f.losses, sizeof(double) * (size_t)s->iters, cudaMemcpyDeviceToHost, st));
    if (grad_norms)
        HG_CUDA(cudaMemcpyAsync(grad_norms, f.losses + s->iters, sizeof(double) * (size_t)s->iters,
                                cudaMemcpyDeviceToHost, st));
    const int src = hg_sync(w);
    if (src == HG_OK && grad_norms)
        for (int it = 0; it < s->iters; ++it) grad_norms[it] = std::sqrt(grad_norms[it]);
    return src;
}

namespace {
struct CkptHeader {
    char magic[8];  // "HGWORLD1"
    uint32_t version;
    int32_t n;
    int32_t layers;
    uint32_t nfields;
    uint64_t step;
    hg_erosion_settings es;
    hg_rain_settings rs;
    uint32_t ks_on;
    hg_step_options opt;
};
const char kCkptMagic[8] = {'H', 'G', 'W', 'O', 'R', 'L', 'D', '1'};
// optional trailer of a particle-mode world: magic, droplet count, the
// droplet arrays (x, y, vx, vy, volume, two sediments, capacity, age, kill),
// then the momentum map's x and y (its z and w are 0 between steps)
const char kPartsMagic[8] = {'H', 'G', 'P', 'A', 'R', 'T', 'S', '1'};
// the nine carried fields, then dirt and dirt sediment (two-layer worlds),
// then the per-cell Ks field when set
std::vector<int> ckpt_fields(int layers, bool ks_on) {
    std::vector<int> f = {HG_FIELD_ROCK,   HG_FIELD_WATER,  HG_FIELD_SEDIMENT, HG_FIELD_FLUX_L, HG_FIELD_FLUX_R,
                          HG_FIELD_FLUX_T, HG_FIELD_FLUX_B, HG_FIELD_VEL_U,    HG_FIELD_VEL_V};
    if (layers == 2) {
        f.push_back(HG_FIELD_DIRT);
        f.push_back(HG_FIELD_SEDIMENT_DIRT);
    }
    if (ks_on) f.push_back(HG_FIELD_KS);
    return f;
}
}  // namespace

int hg_world_save(hg_world* w, const char* path) {
    Range nv_range("hg_world_save");
    HG_CHECK_WORLD(w);
    if (!path) return fail(HG_ERR_INVALID, "null path");
    DeviceGuard g(w->device);
    CkptHeader h{};
    std::memcpy(h.magic, kCkptMagic, 8);
    h.version = 1;
    h.n = w->n;
    h.layers = w->layers;
    const std::vector<int> fields = ckpt_fields(w->layers, w->ks_on);
    h.nfields = (uint32_t)fields.size();
    h.step = w->step;
    h.es = w->es;
    h.rs = w->rs;
    h.ks_on = w->ks_on ? 1 : 0;
    h.opt = w->opt;
    std::vector<float> buf(cells(w));
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(HG_ERR_IO, std::string("cannot open for writing: ") + path);
    bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;
    HG_CUDA(cudaStreamSynchronize(w->stream));
    for (uint32_t k = 0; ok && k < h.nfields; ++k) {
        cudaError_t e =
            cudaMemcpy(buf.data(), field_ptr(w, fields[k]), buf.size() * sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            std::fclose(f);
            return cuda_fail(e, "checkpoint download");
        }
        ok = std::fwrite(buf.data(), sizeof(float), buf.size(), f) == buf.size();
    }
    if (ok && w->parts) {  // particle mode: droplets and the momentum map's x, y
        const Drops& d = w->parts->b.d;
        const int32_t count = d.count;
        ok = std::fwrite(kPartsMagic, 8, 1, f) == 1 && std::fwrite(&count, sizeof(count), 1, f) == 1;
        std::vector<uint32_t> col((size_t)count);
        const void* arrays[10] = {d.px, d.py, d.vx, d.vy, d.vol, d.s0, d.s1, d.sc, d.iters, d.kill};
        for (int k = 0; ok && k < 10; ++k) {
            cudaError_t e = cudaMemcpy(col.data(), arrays[k], col.size() * 4, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) {
                std::fclose(f);
                return cuda_fail(e, "checkpoint download");
            }
            ok = std::fwrite(col.data(), 4, col.size(), f) == col.size();
        }
        for (int k = 0; ok && k < 2; ++k) {
            cudaError_t e =
                cudaMemcpy(buf.data(), w->parts->mom[0][k], buf.size() * sizeof(float), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) {
                std::fclose(f);
                return cuda_fail(e, "checkpoint download");
            }
            ok = std::fwrite(buf.data(), sizeof(float), buf.size(), f) == buf.size();
        }
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return fail(HG_ERR_IO, std::string("write failed: ") + path);
    return HG_OK;
}

int hg_world_load(hg_world* w, const char* path) {
    Range nv_range("hg_world_load");
    HG_CHECK_WORLD(w);
    if (!path) return fail(HG_ERR_INVALID, "null path");
    DeviceGuard g(w->device);
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(HG_ERR_IO, std::string("cannot open: ") + path);
    CkptHeader h{};
    if (std::fread(&h, sizeof(h), 1, f) != 1 || std::memcmp(h.magic, kCkptMagic, 8) != 0 || h.version != 1) {
        std::fclose(f);
        return fail(HG_ERR_IO, std::string("not a world checkpoint: ") + path);
    }
    if (h.n != w->n || h.layers != w->layers) {
        std::fclose(f);
        return fail(HG_ERR_INVALID, "checkpoint world size or layer count differs from this world");
    }
    const std::vector<int> fields = ckpt_fields(h.layers, h.ks_on != 0);
    if (h.nfields != fields.size()) {
        std::fclose(f);
        return fail(HG_ERR_IO, std::string("inconsistent checkpoint header: ") + path);
    }
    std::vector<float> buf(cells(w));
    for (uint32_t k = 0; k < h.nfields; ++k) {
        int field = fields[k];
        if (std::fread(buf.data(), sizeof(float), buf.size(), f) != buf.size()) {
            std::fclose(f);
            return fail(HG_ERR_IO, std::string("truncated checkpoint: ") + path);
        }
        HG_CUDA(cudaMemcpyAsync(field_ptr(w, field), buf.data(), buf.size() * sizeof(float), cudaMemcpyHostToDevice,
                                w->stream));
        HG_CUDA(cudaStreamSynchronize(w->stream));
    }
    char tail[8];
    if (std::fread(tail, 8, 1, f) == 1) {
        int32_t count = 0;
        if (std::memcmp(tail, kPartsMagic, 8) != 0 || std::fread(&count, sizeof(count), 1, f) != 1 || count < 1) {
            std::fclose(f);
            return fail(HG_ERR_IO, std::string("unknown data after the fields: ") + path);
        }
        if (!w->parts || w->parts->count != count) {
            int rc = hg_particles_init(w, count);
            if (rc != HG_OK) {
                std::fclose(f);
                return rc;
            }
        }
        const Drops& d = w->parts->b.d;
        std::vector<uint32_t> col((size_t)count);
        void* arrays[10] = {d.px, d.py, d.vx, d.vy, d.vol, d.s0, d.s1, d.sc, d.iters, d.kill};
        for (int k = 0; k < 12; ++k) {
            const bool field = k >= 10;
            void* dst = field ? (void*)w->parts->mom[0][k - 10] : arrays[k];
            const size_t words = field ? buf.size() : col.size();
            void* src = field ? (void*)buf.data() : (void*)col.data();
            if (std::fread(src, 4, words, f) != words) {
                std::fclose(f);
                return fail(HG_ERR_IO, std::string("truncated checkpoint: ") + path);
            }
            HG_CUDA(cudaMemcpyAsync(dst, src, words * 4, cudaMemcpyHostToDevice, w->stream));
            HG_CUDA(cudaStreamSynchronize(w->stream));
        }
        for (int k = 2; k < 4; ++k) {
            HG_CUDA(cudaMemsetAsync(w->parts->mom[0][k], 0, buf.size() * sizeof(float), w->stream));
        }
        for (int k = 0; k < 4; ++k) HG_CUDA(cudaMemsetAsync(w->parts->mom[1][k], 0, buf.size() * sizeof(float), w->stream));
        HG_CUDA(cudaStreamSynchronize(w->stream));
    }
    std::fclose(f);
    w->step = h.step;
    w->es = h.es;
    w->rs = h.rs;
    w->opt = h.opt;
    w->ks_on = h.ks_on != 0;
    w->dev_step_valid = false;
    w->version += 1;
    w->invalid = false;
    return HG_OK;
}

int hg_selftest_report_timeout(hg_world* w) {
    HG_CHECK_WORLD(w);
    DeviceGuard g(w->device);
    const int one = 1;  // what a kernel's bounded wait writes when it gives up
    HG_CUDA(cudaMemcpyAsync(w->err, &one, sizeof(int), cudaMemcpyHostToDevice, w->stream));
    HG_CUDA(cudaStreamSynchronize(w->stream));
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
