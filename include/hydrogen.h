/* hydrogen.h — C ABI of the GB300 grid-erosion library (libhydrogen_gb300.so).
 *
 * The library replaces hydro-gen's grid-erosion step (the virtual-pipe
 * shallow-water model with hydraulic and thermal erosion) with hand-written
 * CUDA kernels for sm_103a.  Each entry point below names the reference
 * interface it replaces (paths inside the hydro-gen project).
 *
 * Conventions
 *  - Every function returns an int status (HG_OK == 0, negative on error) and
 *    never aborts; hg_last_error() describes the last failure of the calling
 *    thread.
 *  - A world lives on the CUDA device that was current when it was created and
 *    owns one CUDA stream; all work on a world is stream-ordered and
 *    asynchronous unless the function says it synchronises.  A world must not
 *    be used from two host threads at once; distinct worlds may be.
 *  - Fields are n*n float32 arrays, row-major, x fastest; "top" is +y.
 *  - No torch or C++ types cross this boundary: plain pointers and sizes.
 */
#ifndef HYDROGEN_GB300_H
#define HYDROGEN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define HG_OK 0
#define HG_ERR_INVALID (-1)     /* bad argument or settings */
#define HG_ERR_OOM (-2)         /* device or host allocation failed */
#define HG_ERR_CUDA (-3)        /* a CUDA runtime call failed */
#define HG_ERR_TIMEOUT (-4)     /* a bounded device wait gave up */
#define HG_ERR_UNSUPPORTED (-5) /* valid request this build does not support */
#define HG_ERR_IO (-6)          /* checkpoint file error */
#define HG_ERR_STATE (-7)       /* call not valid in the current state */

/* ---- settings ------------------------------------------------------------- */

/* Mirror of Erosion_data (glsl/bindings.glsl:39-60): same field names, order
 * and std140 offsets (96 bytes), so a caller can pass the reference's struct
 * bytes unchanged.  Index [0] is the rock layer, [1] the dirt layer
 * (src/rendering.cpp:214).  Kalpha is the talus angle in radians. */
typedef struct hg_erosion_settings {
    uint32_t particle_count; /*  0  0, or the droplet count of hg_particles_init */
    float Kc;                /*  4  sediment capacity */
    float Kalpha[2];         /*  8  talus angle per layer (radians) */
    float Kconv;             /* 16  rock->dirt sediment conversion */
    float _pad0;             /* 20  std140 alignment of the next vec2 */
    float Ks[2];             /* 24  dissolve (solubility) per layer */
    float Kd[2];             /* 32  deposit per layer */
    float Ke;                /* 40  evaporation */
    float ENERGY_KEPT;       /* 44  flux damping */
    float Kspeed[2];         /* 48  thermal slippage speed per layer */
    float G;                 /* 56  gravity */
    float d_t;               /* 60  time step */
    float density;           /* 64..88 particle-model fields, unused by the grid model */
    float init_volume;
    float friction;
    float inertia;
    float min_volume;
    float min_velocity;
    uint32_t ttl;            /* 88 */
    uint32_t _pad1;          /* 92  std140 struct size is a multiple of 16 */
} hg_erosion_settings;

/* Mirror of Rain_data (glsl/bindings.glsl:62-68), 20 bytes.  The grid step
 * uses `amount` and `period` (rain on step n, 1-based, when n % period == 0,
 * src/main.cpp:315-319); the remaining fields describe the reference's
 * noise-driven rain and are stored unchanged. */
typedef struct hg_rain_settings {
    float amount;
    float mountain_thresh;
    float mountain_multip;
    int32_t period;
    float drops;
} hg_rain_settings;

#define HG_RAIN_OFF 0       /* no rain pass */
#define HG_RAIN_UNIFORM 1   /* every cell gains `amount` */
#define HG_RAIN_REFERENCE 3 /* the reference's rain (glsl/rain.glsl:32-56): amount *
                               max(0, simplex fBm) seeded by the frame time, plus
                               the mountain bonus above mountain_thresh of the map's
                               max_height (hg_set_map_settings) */
#define HG_RAIN_BERNOULLI 2 /* a cell gains `amount` with probability p, drawn
                               from Philox4x32-10 keyed (seed, step, cell) */

#define HG_AUTO (-1)

/* Options of the grid step that the reference fixes in code; kept out of
 * hg_erosion_settings so the 96-byte mirror stays byte-compatible. */
typedef struct hg_step_options {
    int32_t rain_mode;        /* HG_RAIN_* (default HG_RAIN_OFF) */
    float rain_probability;   /* Bernoulli probability per cell and step */
    uint64_t rain_seed;       /* Philox key */
    uint32_t terrain_id;      /* fourth Philox counter word */
    int32_t thermal;          /* HG_AUTO: thermal passes run when Kspeed[0] != 0 */
    int32_t tile_x;           /* fused mode tile width: HG_AUTO or 64 */
    int32_t tile_y;           /* fused mode tile height: HG_AUTO (autotuned), 16 or 8 */
    int32_t graph;            /* fused mode: replay a captured 2-step CUDA graph;
                                 HG_AUTO (autotuned), 0 or 1 */
    float rain_time0;         /* HG_RAIN_REFERENCE: the frame time of step k (1-based) */
    float rain_time_step;     /*   is rain_time0 + k * rain_time_step (seconds) */
    int32_t reserved[4];
} hg_step_options;

/* Map_settings_data (glsl/bindings.glsl:70-99): the reference's terrain
 * generator settings, std140 layout (96 bytes). */
typedef struct hg_map_settings {
    float max_height;
    float max_dirt;
    int32_t hmap_dims[2];
    float height_mult;
    float water_lvl;
    float seed;
    float persistance;
    float lacunarity;
    float scale;
    float redistribution;
    int32_t octaves;
    uint32_t fake_erosion;
    uint32_t mask_round;
    uint32_t mask_exp;
    uint32_t mask_power;
    uint32_t mask_slope;
    uint32_t uplift;
    float uplift_scale;
    int32_t domain_warp;
    float domain_warp_scale;
    int32_t terrace;
    float terrace_scale;
    float _pad0;
} hg_map_settings;

/* Simplex fBm heightmap: octave o samples 2-D simplex noise at cell
 * coordinates times frequency*lacunarity^o with amplitude gain^o and hash
 * seed+o; the sum is min-max scaled to [out_min, out_max]. */
typedef struct hg_noise_settings {
    uint32_t seed;
    int32_t octaves;
    float frequency;
    float lacunarity;
    float gain;
    float out_min;
    float out_max;
} hg_noise_settings;

/* ---- fields ---------------------------------------------------------------- */
#define HG_FIELD_ROCK 0      /* heightmap.r: terrain height */
#define HG_FIELD_WATER 1     /* heightmap.b: water depth */
#define HG_FIELD_SEDIMENT 2  /* sedimap.r: suspended sediment */
#define HG_FIELD_FLUX_L 3    /* fluxmap.x */
#define HG_FIELD_FLUX_R 4    /* fluxmap.y */
#define HG_FIELD_FLUX_T 5    /* fluxmap.z (+y) */
#define HG_FIELD_FLUX_B 6    /* fluxmap.w (-y) */
#define HG_FIELD_VEL_U 7     /* velocitymap.x */
#define HG_FIELD_VEL_V 8     /* velocitymap.y */
#define HG_FIELD_VEL_Z 9     /* velocitymap.z = d1+d2 of the last plain step */
#define HG_FIELD_KS 10       /* per-cell rock solubility (replaces Ks[0]) */
#define HG_FIELD_DIRT 11     /* heightmap.g: dirt layer (two-layer worlds) */
#define HG_FIELD_SEDIMENT_DIRT 12 /* sedimap.g: suspended dirt (two-layer worlds) */
#define HG_FIELD_MOMENTUM_X 13    /* momentmap.x: droplet momentum map (particle mode) */
#define HG_FIELD_MOMENTUM_Y 14    /* momentmap.y */
#define HG_FIELD_COUNT 15

#define HG_MODE_PLAIN 0           /* one kernel per GLSL pass */
#define HG_MODE_FUSED 1           /* fused, tiled kernels: two per step (three in two-layer worlds) */
#define HG_MODE_FUSED_PER_WORLD 2 /* batches only: each world's own fused launches */
#define HG_MODE_PARTICLES 3       /* droplet erosion (hg_particles_init; two-layer worlds) */

typedef struct hg_world hg_world;

/* ---- library ------------------------------------------------------------------ */
const char* hg_version(void);
/* Message of the last failed call on this thread ("" if none). */
const char* hg_last_error(void);

/* Host log hook (no counterpart in the reference, whose LOG / LOG_ERR macros
 * print to stdout, src/utils.hpp:52-66): the library reports every failure
 * (HG_LOG_ERROR, the text hg_last_error returns) and its autotuner's choices
 * (HG_LOG_INFO) by calling fn(level, message, user) on the calling thread.
 * NULL (the default) turns it off.  The message is valid during the call. */
#define HG_LOG_ERROR 0
#define HG_LOG_INFO 1
typedef void (*hg_log_fn)(int level, const char* msg, void* user);
int hg_set_log_callback(hg_log_fn fn, void* user);
/* Number of kernels this library has launched in the process. */
uint64_t hg_launch_count(void);

/* Reference grid-model defaults (src/state.cpp:81-92). */
int hg_default_erosion_settings(hg_erosion_settings* out);
/* Reference particle-model defaults (src/state.cpp:61-79), particle_count 0
 * (hg_set_erosion_settings takes 0 or the world's droplet count). */
int hg_default_particle_settings(hg_erosion_settings* out);
/* Reference rain defaults (src/settings.hpp:16-21). */
int hg_default_rain_settings(hg_rain_settings* out);
int hg_default_step_options(hg_step_options* out);

/* ---- world ------------------------------------------------------------------------- */
/* Replaces State::World::gen_textures (src/state.cpp:3-44): allocates the
 * device fields of an n x n world (n a positive multiple of 8,
 * src/erosion.cpp:83-84) on the current device.  layers 1: rock with an
 * empty dirt layer (Kconv and the dirt layer's terms vanish; every mode);
 * layers 2: the reference's rock + dirt model with both sediment channels
 * (per-pass and fused steps, particle erosion; a batch of them in fused mode
 * runs each world's own fused launches; tapes need layers 1).  All fields
 * start at zero; the settings start at the reference's defaults
 * (src/state.cpp:81-92), with Kconv and Kspeed[1] at 0 for one-layer
 * worlds. */
int hg_world_create(int n, int layers, hg_world** out);

/* The reference's map defaults (src/settings.hpp:27-57) with seed 0 (the
 * reference draws it from rand()). */
int hg_default_map_settings(hg_map_settings* out);
/* Map settings of a world (the rain's mountain bonus reads max_height);
 * "Set Map settings" equivalent. */
int hg_set_map_settings(hg_world* w, const hg_map_settings* s);
/* The reference's terrain generator (glsl/heightmap.glsl:52-158, called by
 * World::gen_heightmap, src/state.cpp:116-147): derivative-damped gradient-
 * noise fBm with domain warp, optional uplift, round/exponential/power/slope
 * masks and terraces; rock = min(max_height, v * max_height * multiplier),
 * dirt = (fBm + 1.5) * max_dirt in two-layer worlds.  Stores the map
 * settings, zeroes water, sediment, flux and velocity, resets the step
 * counter. */
int hg_init_reference_heightmap(hg_world* w, const hg_map_settings* s);
/* The reference's "particle" erosion type (ParticleBuffer, src/state.cpp:28-30;
 * Erosion::dispatch_particle, src/erosion.cpp:132-156): allocates `count`
 * idle droplets (1 <= count <= 2^28) and the momentum map of a two-layer
 * world, or resets them.  hg_step(w, n, HG_MODE_PARTICLES) then runs per
 * step: droplet movement (glsl/particle.glsl:64-136; new droplets spawn
 * while rain_mode != HG_RAIN_OFF, the reference's should_rain), droplet
 * erosion (glsl/particle_erosion.glsl:22-128), the thermal passes of both
 * layers and smoothing with the momentum fold (glsl/smoothing.glsl:22-103).
 * The droplets' updates of a texel apply in droplet-id order (the reference
 * takes a per-texel spinlock in whatever order droplets arrive), and spawn
 * positions come from Philox4x32-10 (counter: droplet id, step, 0x70617274,
 * 0; key: rain_seed) instead of the reference's fract(1e4 sin(...)) hash.
 * The reference dispatches count / work-group-size whole groups; every
 * droplet runs here. */
int hg_particles_init(hg_world* w, int count);
/* Number of droplets (0 before hg_particles_init). */
int hg_particles_count(const hg_world* w, int* count);
/* Droplet state to host memory (any pointer may be NULL): state8 gets 8
 * floats per droplet (x, y, vx, vy, volume, rock sediment, dirt sediment,
 * capacity), iters the age in steps (0: idle), kill 1 for a droplet that
 * respawns on the next step. */
int hg_particles_get(hg_world* w, float* state8, uint32_t* iters, int32_t* kill);
/* Camera of the headless ray-marcher: the uniforms of glsl/rendering.glsl:15-23
 * that Render::Data::dispatch sets (src/rendering.cpp:79-140).  Matrices
 * are column-major as glm stores them. */
typedef struct hg_camera {
    float view[16];          /* glm::lookAt(pos, pos + dir, up) */
    float perspective[16];   /* glm::perspective(radians(FOV), aspect, Z_NEAR, Z_FAR) */
    float pos[3];            /* ray origin (uniform pos) */
    float prec;              /* march step factor (0.35; UI range 0.01..1) */
    int32_t draw_water;      /* should_draw_water (1) */
    int32_t display_sediment;/* tint by suspended sediment (0) */
    float sediment_max_cap;  /* sediment giving full tint (0.1) */
    int32_t low_res_div3;    /* the LOW_RES_DIV3 build: march width/3 x height/3
                                pixels, each stored as a 3x3 block */
} hg_camera;

/* Fills view and perspective as src/rendering.cpp:89-99 does (glm's
 * right-handed lookAt and perspective with depth -1..1) and the other fields
 * with the shader's defaults.  FOV 90, Z_NEAR 0.1, Z_FAR 2048 are the
 * reference's (src/rendering.hpp:11-13). */
int hg_camera_look_at(hg_camera* out, const float pos[3], const float dir[3], const float up[3], float fov_deg,
                      float aspect, float z_near, float z_far);
/* Renders the world into width x height RGBA8 pixels (row y = 0 first, the
 * GL image's bottom row; alpha 0, or 255 in the low-resolution form) and,
 * if rgb is not NULL, the gamma-corrected float colour (3 floats per pixel).
 * hg_render copies into host memory and waits; hg_render_device writes
 * device memory in the world's stream order.  The shader's pow and exp use
 * the library's own exp2 / log2 (GLSL leaves their precision to the driver),
 * so a render is reproducible bit for bit. */
int hg_render(hg_world* w, const hg_camera* cam, int width, int height, uint8_t* rgba, float* rgb);
int hg_render_device(hg_world* w, const hg_camera* cam, int width, int height, uint8_t* rgba_dev, float* rgb_dev);
/* Replaces State::World::delete_textures (src/state.cpp:46-55). */
int hg_world_destroy(hg_world* w);
int hg_world_size(const hg_world* w, int* n);
/* The CUDA stream (cudaStream_t) every call on this world is ordered on. */
int hg_world_stream(const hg_world* w, void** stream);

/* Replaces Erosion_settings::push_data / "Set Erosion settings"
 * (src/settings.hpp:64-66, src/rendering.cpp:303-305).  Takes effect at the
 * next step.  Rejects a particle_count other than 0 or the world's droplet
 * count, d_t <= 0 and, for one-layer worlds, Kconv != 0 (it needs the dirt
 * layer). */
int hg_set_erosion_settings(hg_world* w, const hg_erosion_settings* s);
int hg_get_erosion_settings(const hg_world* w, hg_erosion_settings* s);
/* Replaces Rain_settings::push_data (src/settings.hpp:22-24). */
int hg_set_rain_settings(hg_world* w, const hg_rain_settings* s);
int hg_set_step_options(hg_world* w, const hg_step_options* o);

/* Replaces State::World::gen_heightmap (src/state.cpp:116-147): writes the
 * simplex-fBm heightmap into ROCK, zeroes every other field and resets the
 * step counter. */
int hg_init_heightmap(hg_world* w, const hg_noise_settings* s);
/* Writes a raw (unscaled) fBm field into KS scaled as
 * base * exp(k * fbm / sum_of_amplitudes); used for per-cell solubility. */
int hg_init_ks_field(hg_world* w, const hg_noise_settings* s, float base, float k);
/* Drops the per-cell solubility field (Ks[0] applies again). */
int hg_clear_ks_field(hg_world* w);

/* Starts the world from a caller's heightmap: every field to zero on the
 * device (dirt too in two-layer worlds; the per-cell Ks field stays), then
 * ROCK from caller-owned host memory (n*n floats), step counter 0; the
 * counterpart of creating zero-filled textures (State::World::gen_textures,
 * src/state.cpp:3-44) and writing the heightmap into them.  Synchronous with
 * respect to the host.  HG_ERR_INVALID for a null heightmap. */
int hg_init_heightmap_host(hg_world* w, const float* rock);

/* Copy one field between caller-owned host memory (n*n floats) and the world.
 * Synchronous with respect to the host.  Uploading ROCK or WATER is the
 * equivalent of writing the heightmap texture. */
int hg_world_upload(hg_world* w, int field, const float* host);
int hg_world_download(hg_world* w, int field, float* host);
/* Same with a device pointer (stream-ordered, asynchronous). */
int hg_world_upload_device(hg_world* w, int field, const float* dev);
int hg_world_download_device(hg_world* w, int field, float* dev);

/* Steps completed since the last init (the reference's erosion_steps,
 * src/main.cpp:311). */
int hg_world_get_step(const hg_world* w, uint64_t* step);
int hg_world_set_step(hg_world* w, uint64_t step);

/* ---- the grid step ------------------------------------------------------------------ */
/* Replaces Erosion::dispatch_grid_rain + Erosion::dispatch_grid
 * (src/erosion.hpp:45-46, src/erosion.cpp:76-89, 158-200) called once per
 * main-loop iteration (src/main.cpp:310-320): advances the world by nsteps
 * steps of rain -> hydro_flux -> hydro_erosion -> sediment_transport ->
 * thermal_erosion/thermal_transport.  mode selects the per-pass kernels or
 * the fused kernel; both give bit-identical fields.  Asynchronous. */
int hg_step(hg_world* w, int nsteps, int mode);

/* ---- row slabs (one grid over several GPUs) ------------------------------------------- */
/* No counterpart in the reference, which dispatches every pass over the whole
 * grid (src/erosion.cpp:92-101).  A rank that owns rows of a grid split into
 * row slabs steps them with these, exchanging halo rows between passes (the
 * schedule is hydrogen's slabs.py; its ranks may be processes or threads).
 * hg_set_rows restricts the per-pass kernels to rows [lo, hi) (hi = -1: all
 * rows, the default); while it is set, only one-layer per-pass steps and
 * single passes run (fused steps, batches and tapes are refused with
 * HG_ERR_UNSUPPORTED).  Rows outside the range keep whatever the buffer
 * swaps leave there.  hg_pass runs one pass of the one-layer per-pass step,
 * with that step's operations and buffer swaps: rain uses step number
 * hg_world_get_step + 1 (set it with hg_world_set_step); the talus passes of
 * layer 1 and smoothing with Kspeed[1] == 0 are identities; the reference's
 * rain ignores the row range.  Asynchronous.  hg_world_rows copies rows
 * [y0, y1) of a field between the world and caller-owned host memory (write
 * != 0: into the world), n floats a row, or 4 n for the talus outflow planes
 * (HG_ROWS_THERMAL_C: toward L, R, T, B; HG_ROWS_THERMAL_D: toward LT, RT,
 * LB, RB).  Synchronous with respect to the host. */
#define HG_PASS_RAIN 0
#define HG_PASS_FLUX 1
#define HG_PASS_EROSION 2
#define HG_PASS_SEDIMENT 3
#define HG_PASS_THERMAL_FLUX 4
#define HG_PASS_THERMAL_TRANSPORT 5
#define HG_PASS_SMOOTHING 6
#define HG_ROWS_THERMAL_C 100
#define HG_ROWS_THERMAL_D 101
#define HG_ROWS_ERODED_ROCK 102      /* the fused step's hand-off between its two kernels */
#define HG_ROWS_ERODED_SEDIMENT 103
int hg_set_rows(hg_world* w, int lo, int hi);
int hg_pass(hg_world* w, int pass, int layer);
int hg_world_rows(hg_world* w, int field, int y0, int y1, float* host, int write);
/* One kernel of the fused step over the restricted rows (which 0: rain, flux,
 * erosion, writing the eroded rock and sediment; 1: sediment gather and talus
 * passes, then the step's outputs become the state and the step counter
 * advances).  Between the two, the rows that k_transport reads around a
 * rank's own come from its neighbours: the eroded rock two rows deep and the
 * eroded sediment as deep as the back-traces reach (HG_ROWS_ERODED_*).  For
 * one-layer worlds of sides divisible by 64 without smoothing or the
 * reference's rain; the row range must be whole tile rows (multiples of
 * 16).  Asynchronous. */
int hg_fused_pass(hg_world* w, int which);
/* Replaces Erosion::dispatch_grid_rain (src/erosion.cpp:76-89) for callers
 * that keep the reference's own cadence (src/main.cpp:315-319): one rain
 * pass now, whatever the rain period, with the world's rain model
 * (HG_RAIN_REFERENCE at frame time `time`; uniform and Bernoulli rain keyed
 * by the next step number; nothing when HG_RAIN_OFF).  The step counter does
 * not advance.  Such a caller steps with rain_mode's own cadence disabled
 * (period 0), so hg_step adds no rain of its own.  Asynchronous. */
int hg_rain(hg_world* w, float time);
/* Waits for the world's stream (the reference's glMemoryBarrier/glFinish).
 * HG_ERR_TIMEOUT if a fused-step tile load gave up its bounded wait since the
 * last sync.  After that error the world's fields are undefined: the block
 * that gave up skipped its tile, and a copy it left in flight may still land
 * in shared memory that a later block on the same SM owns, so every world
 * stepped on the same device since the last good sync is suspect too.  The
 * world then refuses hg_step, hg_rain, hg_forward and hg_inverse_fit with
 * HG_ERR_TIMEOUT until hg_init_heightmap, hg_init_reference_heightmap or
 * hg_world_load gives it defined fields again; reload the other worlds of
 * the device from their last checkpoints as well. */
int hg_sync(hg_world* w);
/* Fused-step variant the autotuner chose for this world (tile height 16 or 8,
 * 0 before tuning; graph replay 0/1) and the candidates' ms per step in the
 * order (16, direct), (16, graph), (8, direct), (8, graph).  Tuning happens
 * in the first fused hg_step call of at least 8 steps with tile_y and graph
 * left at HG_AUTO; its steps are ordinary steps (all variants give the same
 * fields). */
int hg_world_tuning(const hg_world* w, int* tile_y, int* graph, double ms[4]);

/* ---- batches of worlds ---------------------------------------------------------------- */
/* No counterpart in the reference (one map per process, src/main.cpp:222).
 * A batch steps several worlds of any sizes (multiples of 64 for the fused
 * mode) and settings together: in HG_MODE_FUSED one launch of each fused
 * kernel covers every tile of every world (a table of per-world descriptors),
 * optionally replayed from a captured CUDA graph; HG_MODE_FUSED_PER_WORLD and
 * HG_MODE_PLAIN run each world's own launches (the one-launch-per-terrain
 * baseline).  The batch has its own stream, ordered after and before the
 * worlds' streams; the worlds stay usable on their own between batch steps. */
typedef struct hg_batch hg_batch;
int hg_batch_create(hg_world* const* worlds, int count, hg_batch** out);
int hg_batch_destroy(hg_batch* b);
int hg_batch_step(hg_batch* b, int nsteps, int mode);
int hg_batch_sync(hg_batch* b);
int hg_batch_stream(const hg_batch* b, void** stream);
int hg_batch_tuning(const hg_batch* b, int* tile_y, int* graph, double ms[4]);
/* Launch form HG_MODE_FUSED chose: with tile_y and graph at HG_AUTO, the first
 * HG_MODE_FUSED call of at least 12 steps also times two steps of every
 * world's own fused launches (4 steps: 2 untimed, 2 timed) and keeps that
 * form when it beat the fastest table launch (per_world 1).  ms_per_world is
 * its ms per step (0 before tuning). */
int hg_batch_launch_form(const hg_batch* b, int* per_world, double* ms_per_world);

/* FP64 totals over the grid, computed on the device:
 * out[0] rock, out[1] water, out[2] sediment.  Synchronises. */
int hg_world_totals(hg_world* w, double out[3]);

/* ---- differentiation ------------------------------------------------------------------ */
/* No counterpart in the reference.  Reverse-mode adjoint of the one-layer
 * step (rain, flux, erosion, sediment transport and, when on, the talus
 * passes; not smoothing), for fitting the per-cell rock solubility and the
 * initial rock heights.  A tape records nsteps steps of w in segments: the
 * first of nsteps - (nseg - 1) * ckpt_every steps, the others of ckpt_every
 * (HG_AUTO: the longest interval whose tape fits in the free device memory
 * less a reserve of a tenth of it, at least 4 GiB; up to nsteps, when
 * nothing is recomputed), with a checkpoint of the carried fields at each
 * segment's start; the last segment stays in the tape, and hg_backward
 * recomputes the others from their checkpoints (nsteps - ckpt_every steps)
 * and runs the reverse kernels.  Subgradients at max/min/clamp and at the
 * dissolve/deposit branches: the taken branch's derivative.  The world's
 * settings and per-cell Ks must not change between hg_forward and
 * hg_backward.  Destroying a world frees the device memory of its live
 * tapes; such a tape then answers HG_ERR_STATE, and hg_tape_destroy only
 * releases its handle. */
typedef struct hg_tape hg_tape;
int hg_tape_create(hg_world* w, int nsteps, int ckpt_every, hg_tape** out);
int hg_tape_destroy(hg_tape* t);
int hg_tape_info(const hg_tape* t, int* nsteps, int* ckpt_every);
/* Advances w by the tape's nsteps fused steps, recording checkpoints. */
int hg_forward(hg_tape* t);
/* Device pointers (n*n floats): dL_drock_final is the loss gradient with
 * respect to the rock field after the recorded steps; outputs (either may be
 * NULL) are the gradients with respect to the per-cell Ks (Ks[0] of every cell
 * when no field is set) and to the rock field before the steps.  Ordered on
 * the world's stream. */
int hg_backward(hg_tape* t, const float* dL_drock_final, float* dL_dks, float* dL_drock0);
/* loss = mean((rock - target)^2) over the grid (FP64 sum) and, if dL_drock is
 * not NULL, its gradient 2*(rock - target)/n^2; target and dL_drock are device
 * pointers.  Synchronises. */
int hg_mse(hg_world* w, const float* target, double* loss, float* dL_drock);

/* Inverse erosion: descent on the per-cell Ks and the initial rock so that
 * the rock after nsteps steps matches a target (the reference has no
 * counterpart; its "Generate" button, src/rendering.cpp:193-202, only runs
 * forward).  Every iteration resets the world to (rock0, no water, sediment,
 * flux or velocity, the step counter of the call), records nsteps fused steps
 * on a tape, takes the MSE loss against the target and its adjoint, and moves
 * each fitted field by a normalised gradient step:
 *   x <- clamp(x - step * g / max|g|, lo, hi)
 * so that no cell changes by more than `step` per iteration. */
typedef struct hg_fit_settings {
    int32_t nsteps;      /* steps per forward */
    int32_t ckpt_every;  /* checkpoint interval, HG_AUTO: the longest that fits */
    int32_t iters;       /* descent iterations (>= 1) */
    float ks_step;       /* largest Ks change per iteration; 0 keeps Ks */
    float ks_min, ks_max;  /* Ks stays in [ks_min, ks_max] */
    float rock_step;     /* largest initial-rock change per iteration; 0 keeps rock0 */
} hg_fit_settings;
int hg_default_fit_settings(hg_fit_settings* out);
/* target, ks and rock0 are device pointers to n*n floats.  ks (in/out, may be
 * NULL when ks_step == 0: the world's Ks then stays) is the starting Ks field
 * and receives the fitted one, which the world also keeps as its Ks field;
 * rock0 (in/out) is the initial rock and receives the fitted one when
 * rock_step > 0.  losses (host, iters doubles) receives the loss of each
 * iteration, taken before its update; grad_norms (host, iters doubles, may
 * be NULL) the L2 norm of that iteration's gradient over the fitted fields
 * (Ks and/or the initial rock), accumulated in FP64 on the device.  The
 * world is left at the end of the
 * last iteration's forward.  The buffers are read and written on the
 * world's stream: work that fills them on other streams must be complete.
 * Same coverage as the tape (one layer, no smoothing).  Synchronises. */
int hg_inverse_fit(hg_world* w, const float* target, float* ks, float* rock0, const hg_fit_settings* s,
                   double* losses, double* grad_norms);

/* ---- checkpoint / resume ------------------------------------------------------------ */
/* No counterpart in the reference (its state lives only in GL textures).
 * Writes the carried fields (rock, water, sediment, four fluxes, u, v; dirt
 * and dirt sediment in two-layer worlds; the per-cell solubility when set),
 * the step counter, the erosion and rain settings and the step options to
 * `path` (a fixed binary header, then little-endian FP32 fields), and in
 * particle mode the droplets and the momentum map.  Resuming with
 * hg_world_load (which sets up the droplets when the file has them) and
 * stepping reproduces an uninterrupted run bit for bit (rain and droplet
 * spawns are keyed by the step counter).  Synchronises.  HG_ERR_IO on file
 * errors, HG_ERR_INVALID if the file's world size or layer count differs
 * from w's. */
int hg_world_save(hg_world* w, const char* path);
int hg_world_load(hg_world* w, const char* path);

/* ---- allocation-free totals -------------------------------------------------------- */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (a host application that owns the device memory budget and lends plugins
 * only its own buffers, or a frame loop that cannot take cudaMalloc's
 * device-wide synchronisation): out[i] = FP64 sum of the `count` floats at
 * device pointer fields[i], for i < nfields <= HG_NOALLOC_MAX_FIELDS, the
 * same reduction as hg_world_totals.  fields is a host array of device
 * pointers; out is device memory for nfields doubles, written on `stream`
 * (a cudaStream_t, NULL for the legacy default stream); asynchronous.
 * Allocates nothing: the partial sums live in a fixed library-global device
 * array of HG_NOALLOC_MAX_FIELDS * 304 doubles (19,456 bytes) that each GPU
 * loading the library holds until the process exits.  Each call looks up
 * that array's address in the current context (so a cudaDeviceReset between
 * calls is harmless); the first call in a context loads the library's module
 * there, so make it before any stream capture in that context.  All calls
 * share the one array: calls whose work overlaps on the
 * GPU (different streams, no ordering between them) race and give wrong
 * sums; order them on one stream or with events.  Rejects nfields outside
 * [1, HG_NOALLOC_MAX_FIELDS] with HG_ERR_INVALID. */
#define HG_NOALLOC_MAX_FIELDS 8
int hg_field_totals_noalloc(const float* const* fields, int nfields, size_t count, double* out, void* stream);

/* ---- self-tests ------------------------------------------------------------------------- */
/* No counterpart in the reference.  Draws `count` operand pairs (seeded) in
 * the range where the fused kernel divides through a shared reciprocal
 * (Markstein's correction) and counts results that differ in any bit from
 * IEEE division; 0 is the only passing answer.  Synchronises. */
int hg_selftest_division(uint64_t seed, uint64_t count, uint64_t* mismatches);
/* The kernels' bounded barrier wait (a TMA tile that never arrives) run on a
 * barrier phase that nothing completes, with no copy in flight: `polls`
 * polls (1 .. 2^18, the kernels' limit), after which the wait gives up.
 * timed_out receives 1 when it did, ns_per_poll the measured time per poll,
 * so 2^18 * ns_per_poll bounds a kernel's wait for a lost tile (about 1 s).  The device
 * stays usable afterwards.  Synchronises. */
int hg_selftest_bounded_wait(uint32_t polls, int* timed_out, double* ns_per_poll);
/* Device self-test of the paired (f32x2) arithmetic the kernels use, lane by
 * lane against the scalar IEEE operations on `count` operand triples drawn
 * from every float bit pattern (subnormals and zeros included):
 * mismatches[0..4] count differing lanes of add, multiply, fused
 * multiply-add, subtract and the shared-reciprocal quotient, mismatches[5]
 * those of a product feeding a sum (which must round twice).  No
 * counterpart in the reference. */
int hg_selftest_paired(uint64_t seed, uint64_t count, uint64_t mismatches[6]);
/* Test hook (no counterpart in the reference): sets the world's device error
 * flag from the host, as a kernel's bounded wait does when it gives up, so
 * that the HG_ERR_TIMEOUT contract of hg_sync can be tested without a GPU
 * fault or a real lost copy. */
int hg_selftest_report_timeout(hg_world* w);
/* Coverage checks.  hg_world_poison_scratch fills every buffer a step writes
 * before reading (the alternate state buffers, velocity, the fused step's
 * hand-off and the thermal scratch; in a world with droplets the droplet
 * records' sediment and layer masks, and not the grid step's velocity,
 * which the particle step leaves alone) with NaN; hg_world_count_nonfinite counts NaN
 * and infinite values over the carried fields (rock, water, sediment, four
 * fluxes, u, v; dirt and dirt sediment in two-layer worlds; the momentum map
 * and the droplets' float state in particle mode).
 * After a step on a poisoned world the count is 0 exactly when the step
 * wrote every cell it owns.  Both are ordered on the world's stream; the
 * count synchronises. */
int hg_world_poison_scratch(hg_world* w);
int hg_world_count_nonfinite(hg_world* w, uint64_t* count);

#ifdef __cplusplus
}
#endif
#endif /* HYDROGEN_GB300_H */
