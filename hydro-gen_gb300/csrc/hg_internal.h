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
// smoothing pass on rock (run when c.smooth_m != 0)
void launch_smooth(const StepConsts& c, const float* rock, float* rock_o, cudaStream_t st);

// ---- the reference's terrain generator and rain (hg_terrain.cu) --------------------
void launch_ref_heightmap(const hg_map_settings& cfg, int n, float* rock, float* dirt, cudaStream_t st);
// water += the reference's rain at frame time `time`; dirt may be nullptr (one layer)
void launch_ref_rain(const hg_rain_settings& rs, const hg_map_settings& map, float time, int n, const float* rock,
                     const float* dirt, float* water, cudaStream_t st);

// ---- two-layer per-pass kernels (hg_layers.cu) -----------------------------------
void launch_flux2(const StepConsts& c, const float* rock, const float* dirt, const float* water, const float* fl,
                  const float* fr, const float* ft, const float* fb, float* water_o, float* fl_o, float* fr_o,
                  float* ft_o, float* fb_o, float* u, float* v, float* vz, cudaStream_t st);
void launch_erosion2(const StepConsts& c, const float* u, const float* v, const float* vz, const float* rock,
                     const float* dirt, float* rock_o, float* dirt_o, float* s0, float* s1, cudaStream_t st);
void launch_sediment2(const StepConsts& c, const float* u, const float* v, const float* s0, const float* s1,
                      float* s0_o, float* s1_o, float* water, cudaStream_t st);
// thermal_erosion for layer 1 (dirt); thermal_transport reuses launch_thermal_in on the dirt field
void launch_thermal_out1(const StepConsts& c, const float* rock, const float* dirt, float4* tc, float4* td,
                         cudaStream_t st);
void launch_smooth2(const StepConsts& c, const float* rock, const float* dirt, float* rock_o, float* dirt_o,
                    cudaStream_t st);

// ---- headless ray-marcher (hg_render.cu) ------------------------------------------
struct RenderInput {
    int n;
    float max_height;  // map settings: the shadow rays' ceiling
    int hmap_dim_x;    // map settings: alpha of the low-resolution form
    const float* rock;
    const float* dirt;   // nullptr: one-layer world
    const float* water;
    const float* sed0;
    const float* sed1;   // nullptr: one-layer world
    float4* hm;          // n*n packed heightmap texels (written)
    float2* sed;         // n*n packed sediment texels (written when displayed)
};
// packs the heightmap and renders width x height pixels into rgba_dev
// (and the float colour into rgb_dev when not null); HG_ERR_INVALID for a
// singular view or perspective matrix
int render_image(const RenderInput& in, const hg_camera& cam, int width, int height, uint8_t* rgba_dev,
                 float* rgb_dev, cudaStream_t st);

// ---- fused two-layer step (hg_fused2.cu) ------------------------------------------
// Inputs and outputs of one fused two-layer step (out of place) and its
// scratch fields.
struct Fused2Bufs {
    const float *rock, *dirt, *water, *s0, *s1, *fl, *fr, *ft, *fb;
    float *rock_o, *dirt_o, *water_o, *s0_o, *s1_o, *fl_o, *fr_o, *ft_o, *fb_o;
    float *u, *v;
    float *s0_ero, *s1_ero;  // eroded sediment (rock, dirt)
    float *b_ero;            // eroded rock (input of the rock talus pass)
    float *rock_mid;         // rock after the rock talus pass (input of the dirt pass)
    float *g_ero;            // eroded dirt (input of the dirt pass)
};
struct TmaCache;
bool fused2_ok(int n);
int launch_fused2_step(const StepConsts& c, const Talus1& t1, const RainStep& r, const Fused2Bufs& b, TmaCache& tma,
                       int* err, cudaStream_t st);

// ---- particle erosion (hg_particles.cu) --------------------------------------------
// Droplets as structure of arrays (Particle, glsl/bindings.glsl:101-110).
struct Drops {
    int count;
    float *px, *py, *vx, *vy, *vol;
    float *s0, *s1;  // sediment of the rock / dirt layer
    float* sc;       // sediment capacity
    uint32_t* iters;
    int32_t* kill;
};
// Counting-sort and per-record buffers of one particle world.
struct ParticleBufs {
    Drops d;
    uint32_t* cnt;         // n*n records per texel
    uint32_t* offs;        // n*n + 1 exclusive prefix
    uint32_t* cursor;      // n*n scatter cursors
    uint32_t* block_sums;  // particle_scan_blocks(n*n)
    uint32_t* keys;        // 4*count records (droplet * 4 + corner), bucketed by texel
    uint32_t* sorted;      // 4*count: hot texels' buckets in droplet-id order
    uint32_t* hot;         // 2 + 2*hot_cap: counts of mid and big texels, then their indices
    uint32_t hot_cap;      // particle_hot_capacity(n*n, count)
    float* rec;            // 8*count: per record the dirt and rock sediment it left
    uint8_t* rec_mask;     // 4*count: which layers a record set
};
// The fields a particle pass reads or writes; mom = momentum (x, y, z, w).
struct PWorld {
    float* rock;
    float* dirt;
    float* water;
    float* mom[4];
};
size_t particle_scan_blocks(size_t cells);
size_t particle_hot_capacity(size_t cells, int count);
// movement, counting sort, erosion in droplet-id order, sediment replay
void launch_particle_step(const StepConsts& c, const hg_erosion_settings& es, const ParticleBufs& pb,
                          const PWorld& pw, uint32_t step1, uint64_t seed, bool should_rain, cudaStream_t st);
// smoothing with the particle branch: in -> out (all of rock, dirt, water, momentum)
void launch_particle_smooth(const StepConsts& c, float count, const PWorld& in, const PWorld& out, cudaStream_t st);
struct TmaCache;
struct Talus1;
// the particle step's talus passes (rock, then dirt) and smoothing with the
// particle branch as fused kernels (hg_fused2.cu, n a multiple of 64):
// in -> out, the rock after its talus pass in rock_mid
int launch_particle_thermal_smooth(const StepConsts& c, const Talus1& t1, float count, const PWorld& in,
                                   const PWorld& out, float* rock_mid, TmaCache& tma, int* err, cudaStream_t st);

// ---- fused step (hg_fused.cu) ---------------------------------------------------
// Rain settings without the step number (the kernels add the step).
struct RainBase {
    int mode;  // HG_RAIN_*
    int period;
    float amount;
    uint32_t threshold;
    uint32_t seed_lo, seed_hi, terrain_id;
};

// One terrain (world) of a fused launch, without its tensor maps.
struct TerrainHot {
    StepConsts c;
    RainBase rain;
    float* out[S_COUNT];
    float* u;
    float* v;
    float* s_ero;  // eroded sediment of every cell (k_hydro -> k_transport)
    float* b_ero;  // eroded rock of every cell (k_hydro -> k_transport, thermal on)
    unsigned long long* step;  // device step counter (steps completed)
    int tiles_x;
    int tile0;  // first tile of this terrain in the launch
};
// maps[0..6]: TMA boxes of the step's input rock, water, sediment, fL, fR,
// fT, fB; maps[7]: eroded rock.  (CUtensorMap makes it 64-byte aligned.)
constexpr int MAPS_PER_TERRAIN = 8;
struct TerrainDesc {
    CUtensorMap maps[MAPS_PER_TERRAIN];
    TerrainHot h;
    int tile_off;  // first tile launched (a row slab's), 0 for the whole world
};
// A batch launch's terrain records travel as one kernel parameter (read
// through the constant bank); the tensor maps stay in global memory.
constexpr int MAX_BATCH = 128;
struct BatchParams {
    int nterr;
    int tile0[MAX_BATCH];
    TerrainHot t[MAX_BATCH];
};
static_assert(sizeof(BatchParams) < 32000, "kernel parameter space");

// Host view of one terrain for one step direction (inputs -> outputs).
struct TerrainSrc {
    StepConsts c;
    RainBase rain;
    const float* in[S_COUNT];
    float* out[S_COUNT];
    float* u;
    float* v;
    float* s_ero;
    float* b_ero;
    unsigned long long* step;
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

// Tile height th (16 or 8) divides n and 64 divides n.
bool fused_tile_ok(int n, int th);
int fused_tiles(int n, int th);
// Fills a descriptor (tensor maps from the cache); false if a map cannot be encoded.
bool fill_desc(TerrainDesc& d, const TerrainSrc& s, int th, int tile0, TmaCache& cache);
// k_hydro then k_transport over every tile of the batch's terrains; maps
// holds MAPS_PER_TERRAIN tensor maps per terrain (device memory).
void launch_fused_table(const BatchParams& bp, const CUtensorMap* maps, int total_tiles, int th, int* err,
                        cudaStream_t st);
// Same for one terrain whose descriptor travels as a kernel parameter.
void launch_fused_one(const TerrainDesc& td, int th, int* err, cudaStream_t st);
// One kernel of the fused step (which 0: k_hydro, 1: k_transport) over tiles
// [tile_lo, tile_lo + tiles) of a single world.
void launch_fused_half(const TerrainDesc& td, int th, int which, int tile_lo, int tiles, int* err, cudaStream_t st);

// ---- adjoint (hg_adjoint.cu) ----------------------------------------------------------
// A step's state or its adjoint: rock, water, sediment, fL, fR, fT, fB.
struct AdjFields {
    float* b;
    float* d;
    float* s;
    float* f[4];
};
// Forward intermediates of one step kept by the segment recompute.
struct AdjSlot {
    const float* u;
    const float* v;
    const float* se;  // eroded sediment
};
// packet fields of a state adjoint: height-difference terms toward L, R, T,
// B, inflow terms from L, R, T, B, terrain-normal x and z terms
constexpr int ADJ_PACKET_FIELDS = 10;
// Adjoint of a state: each cell's own terms (rock, water, fluxes) plus the
// packets of the terms of its neighbours' inputs; the sediment adjoint needs
// no packets.
struct AdjView {
    const float* b;
    const float* d;
    const float* f[4];
    const float* pdh[4];
    const float* pin[4];
    const float* pdx;
    const float* pdz;
};
// Arguments of k_adj_cell (one kernel parameter).
struct AdjCellArgs {
    CUtensorMap maps[7];  // X: rock, water, sediment, fL, fR, fT, fB (64-wide tiles, 1-cell halo)
    StepConsts c;
    RainStep rain;
    AdjView A;            // adjoint of the step's output
    float* dse;           // this step's sediment adjoint (read, then cleared)
    float* dse_prev;      // step j - 1's sediment adjoint (scatter target)
    float* du;            // back-trace velocity adjoint: read for step j, written for step j - 1
    float* dv;
    const float* gbe;     // thermal on: adjoint of the eroded rock (replaces A's rock), else nullptr
    AdjSlot prev;         // step j - 1's intermediates
    int scatter_prev;     // reverse step j - 1's sediment pass here (its intermediates exist)
    float* rb;            // R: own terms of the input adjoint
    float* rd;
    float* rs;
    float* rf[4];
    float* pdh[4];        // R: packets
    float* pin[4];
    float* pdx;
    float* pdz;
    float* dks;           // per-cell Ks gradient (accumulated)
};
bool adjoint_tile_ok(int n);
// Rows of the TMA box k_adj_cell stages per field (tile rows plus halo);
// AdjCellArgs::maps must be encoded with this box height.
int adjoint_box_rows();
void launch_adjoint_sediment(const StepConsts& c, const AdjSlot& slot, const float* as, float* dse, float* du,
                             float* dv, cudaStream_t st);
void launch_adjoint_cell(const AdjCellArgs& args, int* err, cudaStream_t st);
// gathered rock adjoint of a state into out_b
void launch_adjoint_final(int n, const AdjView& A, float* out_b, cudaStream_t st);
// reverse of the talus passes: A (adjoint of the step's output, own terms and
// packets; its rock part is gathered in the kernel) -> g (adjoint of the
// eroded rock); map_b: boxes 72 x adjoint_thermal_box_rows() of the eroded rock
int adjoint_thermal_box_rows();
void launch_adjoint_thermal(const StepConsts& c, const CUtensorMap& map_b, const AdjView& A, float* g, int* err,
                            cudaStream_t st);
// loss = mean((b - target)^2) into *out (device), grad = dloss/db (optional).
void launch_mse(const float* b, const float* target, size_t count, float* grad, double* part, int nparts,
                double* out, cudaStream_t st);
// *out += the count of NaN and infinite values of x
void launch_count_nonfinite(const float* x, size_t count, unsigned long long* out, cudaStream_t st);
// *out += sum of g^2 in FP64 (fixed order); part holds nparts doubles
void launch_add_sumsq(const float* g, size_t count, double* part, int nparts, double* out, cudaStream_t st);
// x <- clamp(x - step * g / max|g|, lo, hi); part holds nparts floats
void launch_descend(float* x, const float* g, size_t count, float step, float lo, float hi, float* part, int nparts,
                    cudaStream_t st);

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
