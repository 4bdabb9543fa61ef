// Particle (droplet) erosion, src/erosion.cpp:132-156: movement
// (glsl/particle.glsl:64-136), erosion (glsl/particle_erosion.glsl:22-128),
// the thermal passes and smoothing with its particle branch
// (glsl/smoothing.glsl:22-103).
//
// The shader serialises the droplets' updates of a texel with a spinlock per
// texel, in whatever order the droplets win it.  Here the order is fixed and
// no thread waits on another:
//   k_pcount / scan / k_pscatter   counting sort of the droplets' four corner
//                                  records by texel
//   k_papply / _mid / _big         each texel applies its records in
//                                  droplet-id order (a texel update needs only
//                                  the droplet's state from before the pass)
//                                  and stores what each corner left for the
//                                  droplet's sediment; a texel with up to 8
//                                  records sorts them in its thread's
//                                  registers, up to 32 across a warp's lanes,
//                                  more in a warp's shared memory
//   k_pfinal                       each droplet replays its corners 0..3
// which is a sequential pass over droplets in id order, corners in order.
// Spawn positions come from Philox4x32-10 (counter: droplet id, step,
// 'part', 0; key: the rain seed), 24-bit uniforms; the shader's
// fract(1e4 sin(...)) hash of the frame time has no portable bits.
#include "hg_internal.h"

#include <algorithm>

namespace hg {

namespace {

constexpr int BX = 32, BY = 8, PB = 256;

__device__ __forceinline__ float fract_(float x) { return x - floorf(x); }
__device__ __forceinline__ bool inb(int n, int x, int y) { return x >= 0 && x < n && y >= 0 && y < n; }

// img_bilinear (glsl/img_interpolation.glsl:3-22) of a field, 0 outside
__device__ __forceinline__ float bilin(const float* f, int n, float sx, float sy) {
    const int ix = (int)sx, iy = (int)sy;
    const float fx = fract_(sx), fy = fract_(sy);
    auto t = [&](int xx, int yy) { return inb(n, xx, yy) ? f[(size_t)yy * n + xx] : 0.0f; };
    const float v1 = gmix(t(ix, iy), t(ix + 1, iy), fx);
    const float v2 = gmix(t(ix, iy + 1), t(ix + 1, iy + 1), fx);
    return gmix(v1, v2, fy);
}

struct MoveArgs {
    StepConsts c;
    hg_erosion_settings es;
    Drops d;
    const float* rock;
    const float* dirt;
    const float* water;
    const float* mx;
    const float* my;
    uint32_t step1;
    uint32_t seed_lo, seed_hi;
    int should_rain;
};

__global__ void k_pmove(const MoveArgs a) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= a.d.count) return;
    const int n = a.c.n;
    const float dt = a.es.d_t;
    uint32_t iters = a.d.iters[id];
    int kill = a.d.kill[id];
    if (iters == 0 && !a.should_rain) return;
    float px = a.d.px[id], py = a.d.py[id], vx = a.d.vx[id], vy = a.d.vy[id], vol = a.d.vol[id];
    float s0 = a.d.s0[id], s1 = a.d.s1[id], sc = a.d.sc[id];
    if (s0 < 0.0f || iters == 0) s0 = 0.0f;
    if (s1 < 0.0f || iters == 0) s1 = 0.0f;
    bool done = false;
    if (iters == 0 || kill) {
        uint32_t w[4] = {(uint32_t)id, a.step1, 0x70617274u, 0u};
        philox4x32_10(w, a.seed_lo, a.seed_hi);
        const float span = (float)n - 4.0f;
        kill = 0;
        px = (float)(w[0] >> 8) * 0x1p-24f * span / 1.0f + 2.0f;
        py = (float)(w[1] >> 8) * 0x1p-24f * span / 1.0f + 2.0f;
        vx = 0.0f;
        vy = 0.0f;
        vol = a.es.init_volume;
        iters = a.should_rain ? 1u : 0u;
        done = !a.should_rain;
    }
    if (!done) {
        // get_terr_normal (:48-60)
        const float rr = bilin(a.rock, n, px + 1.0f, py), rg = bilin(a.dirt, n, px + 1.0f, py);
        const float lr = bilin(a.rock, n, px - 1.0f, py), lg = bilin(a.dirt, n, px - 1.0f, py);
        const float br = bilin(a.rock, n, px, py - 1.0f), bg = bilin(a.dirt, n, px, py - 1.0f);
        const float tr = bilin(a.rock, n, px, py + 1.0f), tg = bilin(a.dirt, n, px, py + 1.0f);
        const float dx = rr + rg - lr - lg;
        const float dz = tr + tg - br - bg;
        const float cx = dx * 2.0f - 0.0f * dz, cy = 0.0f * 0.0f - 2.0f * 2.0f, cz = 2.0f * dz - dx * 0.0f;
        const float len = sqrtf(cx * cx + cy * cy + cz * cz);
        const float nx = cx / len, ny = cy / len, nz = cz / len;
        const float mxv = bilin(a.mx, n, px, py), myv = bilin(a.my, n, px, py);
        const float water = bilin(a.water, n, px, py);
        vx -= (dt * nx) / vol * a.es.G;
        vy -= (dt * nz) / vol * a.es.G;
        const float lm = sqrtf(mxv * mxv + myv * myv);
        float lv = sqrtf(vx * vx + vy * vy);
        if (lm > 0.0f && lv > 0.0f) {
            const float d = (mxv / lm) * (vx / lv) + (myv / lm) * (vy / lv);
            const float k = a.es.inertia * d / (vol + 1e5f * water);
            vx += k * mxv;
            vy += k * myv;
        }
        lv = sqrtf(vx * vx + vy * vy);
        if (lv > 1.0f) {  // capped speed: no tunnelling through the terrain
            vx = vx / lv;
            vy = vy / lv;
        }
        const float ox = px, oy = py;
        px += dt * vx;
        py += dt * vy;
        if (px <= 1.0f || py <= 1.0f || px * 1.0f >= (float)(n - 2) || py * 1.0f >= (float)(n - 2)) {
            px = ox; py = oy; vx = 0.0f; vy = 0.0f; kill = 1;
        }
        const float fr = 1.0f - dt * a.es.friction * ny;
        vx *= fr;
        vy *= fr;
        vol -= dt * a.es.Ke;
        const float sin_a = fabsf(sqrtf(1.0f - ny * ny));
        lv = sqrtf(vx * vx + vy * vy);
        sc = gmax(0.0f, a.es.Kc * vol * lv * gmax(0.02f, sin_a));
        iters++;
        if (vol <= a.es.min_volume || lv < a.es.min_velocity || iters >= a.es.ttl) kill = 1;
    }
    a.d.px[id] = px; a.d.py[id] = py; a.d.vx[id] = vx; a.d.vy[id] = vy; a.d.vol[id] = vol;
    a.d.s0[id] = s0; a.d.s1[id] = s1; a.d.sc[id] = sc; a.d.iters[id] = iters; a.d.kill[id] = kill;
}

// corner k of a droplet: texel (cx, cy) and weight.  A live droplet sits in
// (1, n - 2) on both axes (movement reverts steps that leave it), so the
// clamp only keeps a non-finite position's texels inside the map.
__device__ __forceinline__ void corner(float px, float py, int k, int n, int& cx, int& cy, float& wgt) {
    const int bx = min(max((int)(px * 1.0f), 0), n - 2), by = min(max((int)(py * 1.0f), 0), n - 2);
    const float ofx = fract_(px * 1.0f), ofy = fract_(py * 1.0f);
    cx = (k == 1 || k == 2) ? bx + 1 : bx;
    cy = (k >= 2) ? by + 1 : by;
    const float wx = (k == 1 || k == 2) ? ofx : 1.0f - ofx;
    const float wy = (k >= 2) ? ofy : 1.0f - ofy;
    wgt = wx * wy;
}

__global__ void k_pcount(Drops d, int n, uint32_t* __restrict__ cnt) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= d.count || d.iters[id] == 0) return;
    for (int k = 0; k < 4; ++k) {
        int cx, cy;
        float wgt;
        corner(d.px[id], d.py[id], k, n, cx, cy, wgt);
        atomicAdd(cnt + (size_t)cy * n + cx, 1u);
    }
}

__global__ void k_pscatter(Drops d, int n, uint32_t* __restrict__ cursor, uint32_t* __restrict__ keys) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= d.count || d.iters[id] == 0) return;
    for (int k = 0; k < 4; ++k) {
        int cx, cy;
        float wgt;
        corner(d.px[id], d.py[id], k, n, cx, cy, wgt);
        const uint32_t slot = atomicAdd(cursor + (size_t)cy * n + cx, 1u);
        keys[slot] = (uint32_t)id * 4u + (uint32_t)k;
    }
}

// exclusive scan of up to 4096 x 4096 counts: blocks of 4096, then the block sums
constexpr int SCAN_T = 1024, SCAN_E = 4;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums, uint32_t& total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warp_sums[lane] = s;  // inclusive
    }
    __syncthreads();
    total = warp_sums[(blockDim.x >> 5) - 1];
    const uint32_t before = wid > 0 ? warp_sums[wid - 1] : 0u;
    return before + x - v;
}

__global__ void k_scan_blocks(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, size_t count,
                              uint32_t* __restrict__ block_sums) {
    __shared__ uint32_t ws[32];
    const size_t base = (size_t)blockIdx.x * SCAN_T * SCAN_E + (size_t)threadIdx.x * SCAN_E;
    uint32_t v[SCAN_E], sum = 0;
#pragma unroll
    for (int e = 0; e < SCAN_E; ++e) {
        v[e] = base + e < count ? in[base + e] : 0u;
        sum += v[e];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan(sum, ws, total);
#pragma unroll
    for (int e = 0; e < SCAN_E; ++e) {
        if (base + e < count) out[base + e] = run;
        run += v[e];
    }
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// one block: exclusive scan of the block sums in place, chunk by chunk; grand total into *total_out
__global__ void k_scan_sums(uint32_t* __restrict__ sums, int nb, uint32_t* __restrict__ total_out) {
    __shared__ uint32_t ws[32];
    uint32_t carry = 0;
    for (int chunk = 0; chunk < nb; chunk += SCAN_T * SCAN_E) {
        const int base = chunk + threadIdx.x * SCAN_E;
        uint32_t v[SCAN_E], sum = 0;
#pragma unroll
        for (int e = 0; e < SCAN_E; ++e) {
            v[e] = base + e < nb ? sums[base + e] : 0u;
            sum += v[e];
        }
        uint32_t total;
        uint32_t run = carry + block_exclusive_scan(sum, ws, total);
#pragma unroll
        for (int e = 0; e < SCAN_E; ++e) {
            if (base + e < nb) sums[base + e] = run;
            run += v[e];
        }
        carry += total;
        __syncthreads();  // ws is reused by the next chunk
    }
    if (threadIdx.x == 0) *total_out = carry;
}

__global__ void k_scan_add(uint32_t* __restrict__ out, uint32_t* __restrict__ cursor, size_t count,
                           const uint32_t* __restrict__ sums) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint32_t v = out[i] + sums[i / (SCAN_T * SCAN_E)];
    out[i] = v;
    cursor[i] = v;
}

struct ApplyArgs {
    hg_erosion_settings es;
    Drops d;
    int n;
    const uint32_t* offs;  // n*n + 1
    uint32_t* keys;        // records bucketed by texel, any order within a bucket
    uint32_t* sorted;      // big texels: their bucket in droplet-id order
    uint32_t* hot;         // [0], [1]: mid and big texel counts; then mid texels
                           // from [2], big texels from [2 + hot_cap]
    uint32_t hot_cap;
    float* rock;
    float* dirt;
    float* water;
    float* mz;
    float* mw;
    float* rec;            // per record (droplet * 4 + corner): s1 of dirt, s1 of rock
    uint8_t* rec_mask;     // bit 1: dirt layer handled, bit 0: rock layer handled
};

// A record's inputs: all from before the pass
struct Rec {
    uint32_t key;
    float multipl, sc, vol, s0, s1, vx, vy;
    int kill;
};

__device__ __forceinline__ Rec load_rec(const ApplyArgs& a, uint32_t key) {
    Rec r;
    r.key = key;
    const int id = (int)(key >> 2), k = (int)(key & 3u);
    int cx, cy;
    corner(a.d.px[id], a.d.py[id], k, a.n, cx, cy, r.multipl);
    r.sc = a.d.sc[id];
    r.vol = a.d.vol[id];
    r.s0 = a.d.s0[id];
    r.s1 = a.d.s1[id];
    r.vx = a.d.vx[id];
    r.vy = a.d.vy[id];
    r.kill = a.d.kill[id];
    return r;
}

struct Texel {
    float terr[2], wat, mz, mw;
};

// what a record leaves for its droplet's sediment replay
struct RecOut {
    float s_dirt, s_rock;
    uint32_t mask;
};

// one droplet corner on its texel (glsl/particle_erosion.glsl:66-122): the
// layer loop from dirt down to rock, then water and momentum
__device__ __forceinline__ RecOut apply_record(const ApplyArgs& a, const Rec& r, Texel& T) {
    const float old_sed[2] = {r.s0, r.s1};
    float s_out[2] = {0.0f, 0.0f};
    uint32_t mask = 0;
    float cap = 0.0f;
    for (int l = 1; l >= 0; --l) {
        if (r.kill) {
            T.terr[l] += old_sed[l] * r.multipl;
            continue;
        }
        const float Kls = a.es.d_t * a.es.Ks[l], Kld = a.es.d_t * a.es.Kd[l];
        const float c = gmax(0.0f, r.sc - cap);
        float s1 = old_sed[l];
        const float old_terr = T.terr[l];
        mask |= 1u << l;
        if (c > s1) {
            const float eroded = r.multipl * Kls * (c - s1);
            s1 += eroded;
            T.terr[l] -= eroded;
            if (T.terr[l] < 0.0f) {
                s1 += T.terr[l];
                T.terr[l] = 0.0f;
                cap += old_terr;
            } else {
                s_out[l] = s1;
                break;
            }
        } else {
            const float deposit = r.multipl * Kld * (s1 - c);
            s1 -= deposit;
            T.terr[l] += deposit;
        }
        s_out[l] = s1;
    }
    T.wat += 1e-5f * r.vol * r.multipl;
    T.mz += r.vol * r.vx * r.multipl;
    T.mw += r.vol * r.vy * r.multipl;
    return RecOut{s_out[1], s_out[0], mask};
}

// A record's update with its texel-independent parts computed ahead (in
// parallel across a warp's lanes): the dirt step with no layer exhausted,
// then the rock step.  mode 0: kill (both layers take their share back);
// 1: dirt dissolves and the loop breaks; 2: dirt deposits, rock dissolves;
// 3: both deposit.  Only an exhausted dirt layer (mode 1 going below zero)
// needs the full update, apply_record.
struct Pre {
    uint32_t key;
    int mode;
    float d1, d0;    // kill: the returned sediment; else the dissolved / deposited amounts
    float s1n, s0n;  // the dirt / rock sediment after their step
    float wi, mzi, mwi;
};

__device__ __forceinline__ Pre prep_record(const ApplyArgs& a, const Rec& r) {
    Pre p;
    p.key = r.key;
    p.wi = 1e-5f * r.vol * r.multipl;
    p.mzi = r.vol * r.vx * r.multipl;
    p.mwi = r.vol * r.vy * r.multipl;
    p.s1n = 0.0f;
    p.s0n = 0.0f;
    if (r.kill) {
        p.mode = 0;
        p.d1 = r.s1 * r.multipl;
        p.d0 = r.s0 * r.multipl;
        return p;
    }
    const float c = gmax(0.0f, r.sc - 0.0f);  // cap is 0 until a layer is exhausted
    if (c > r.s1) {
        p.mode = 1;
        p.d1 = r.multipl * (a.es.d_t * a.es.Ks[1]) * (c - r.s1);
        p.s1n = r.s1 + p.d1;
        p.d0 = 0.0f;
        return p;
    }
    p.d1 = r.multipl * (a.es.d_t * a.es.Kd[1]) * (r.s1 - c);
    p.s1n = r.s1 - p.d1;
    if (c > r.s0) {
        p.mode = 2;
        p.d0 = r.multipl * (a.es.d_t * a.es.Ks[0]) * (c - r.s0);
        p.s0n = r.s0 + p.d0;
    } else {
        p.mode = 3;
        p.d0 = r.multipl * (a.es.d_t * a.es.Kd[0]) * (r.s0 - c);
        p.s0n = r.s0 - p.d0;
    }
    return p;
}

// the texel-dependent rest of a prepared record; false (texel untouched)
// when the dirt layer would be exhausted
__device__ __forceinline__ bool apply_prepared(const Pre& p, Texel& T, RecOut& o) {
    if (p.mode == 1) {
        const float t = T.terr[1] - p.d1;
        if (t < 0.0f) return false;
        T.terr[1] = t;
        o = RecOut{p.s1n, 0.0f, 2u};
    } else if (p.mode == 0) {
        T.terr[1] += p.d1;
        T.terr[0] += p.d0;
        o = RecOut{0.0f, 0.0f, 0u};
    } else if (p.mode == 2) {
        T.terr[1] += p.d1;
        const float t = T.terr[0] - p.d0;
        if (t < 0.0f) {
            o = RecOut{p.s1n, p.s0n + t, 3u};
            T.terr[0] = 0.0f;
        } else {
            o = RecOut{p.s1n, p.s0n, 3u};
            T.terr[0] = t;
        }
    } else {
        T.terr[1] += p.d1;
        T.terr[0] += p.d0;
        o = RecOut{p.s1n, p.s0n, 3u};
    }
    T.wat += p.wi;
    T.mz += p.mzi;
    T.mw += p.mwi;
    return true;
}

__device__ __forceinline__ void store_rec(const ApplyArgs& a, uint32_t key, const RecOut& o) {
    a.rec[2 * key + 0] = o.s_dirt;
    a.rec[2 * key + 1] = o.s_rock;
    a.rec_mask[key] = (uint8_t)o.mask;
}

__device__ __forceinline__ Texel load_texel(const ApplyArgs& a, size_t t) {
    return Texel{{a.rock[t], a.dirt[t]}, a.water[t], a.mz[t], a.mw[t]};
}
__device__ __forceinline__ void store_texel(const ApplyArgs& a, size_t t, const Texel& T) {
    a.rock[t] = T.terr[0];
    a.dirt[t] = T.terr[1];
    a.water[t] = T.wat;
    a.mz[t] = T.mz;
    a.mw[t] = T.mw;
}

constexpr int SMALL = 8;  // records a texel's own thread sorts and applies
constexpr int MID = 32;   // records a warp sorts in registers

// each texel with at most SMALL records applies them in droplet-id order;
// busier texels go to the mid (up to MID records) or big lists
__global__ void k_papply(const ApplyArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = a.n;
    if (x >= n || y >= n) return;
    const size_t t = (size_t)y * n + x;
    const uint32_t lo = a.offs[t], hi = a.offs[t + 1];
    if (lo == hi) return;
    const uint32_t k = hi - lo;
    if (k > SMALL) {
        const int big = k > (uint32_t)MID ? 1 : 0;
        const uint32_t slot = atomicAdd(a.hot + big, 1u);
        if (slot < a.hot_cap) a.hot[2 + big * a.hot_cap + slot] = (uint32_t)t;
        return;
    }
    uint32_t kk[SMALL];
#pragma unroll
    for (int i = 0; i < SMALL; ++i) kk[i] = (uint32_t)i < k ? a.keys[lo + i] : 0xffffffffu;
    // sorting network on registers (odd-even transposition, SMALL rounds)
#pragma unroll
    for (int r = 0; r < SMALL; ++r)
#pragma unroll
        for (int i = r & 1; i + 1 < SMALL; i += 2) {
            const uint32_t u = min(kk[i], kk[i + 1]), v = max(kk[i], kk[i + 1]);
            kk[i] = u;
            kk[i + 1] = v;
        }
    Texel T = load_texel(a, t);
#pragma unroll
    for (int i = 0; i < SMALL; ++i)
        if ((uint32_t)i < k) store_rec(a, kk[i], apply_record(a, load_rec(a, kk[i]), T));
    store_texel(a, t, T);
}

constexpr int HOT_WARPS = 4;     // warps per block of the mid / big kernels
constexpr int HOT_KEYS = 2048;   // bucket size a warp sorts in shared memory

// one warp per mid texel (SMALL < records <= 32): lane i holds record i;
// a bitonic network over the lanes sorts the keys by droplet id, each lane
// loads its record, and the warp runs the texel's sequential update in
// lockstep with record i's prepared update broadcast from lane i
__global__ void __launch_bounds__(32 * HOT_WARPS) k_papply_mid(const ApplyArgs a) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const uint32_t nmid = min(a.hot[0], a.hot_cap);
    for (uint32_t h = blockIdx.x * HOT_WARPS + wl; h < nmid; h += gridDim.x * HOT_WARPS) {
        const size_t t = a.hot[2 + h];
        const uint32_t lo = a.offs[t], k = a.offs[t + 1] - lo;
        uint32_t key = (uint32_t)lane < k ? a.keys[lo + lane] : 0xffffffffu;
#pragma unroll
        for (int size = 2; size <= 32; size <<= 1)
#pragma unroll
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                const uint32_t other = __shfl_xor_sync(FULL, key, stride);
                const bool up = (lane & size) == 0, lower = (lane & stride) == 0;
                key = (lower == up) ? min(key, other) : max(key, other);
            }
        Rec mine{};
        if ((uint32_t)lane < k) mine = load_rec(a, key);
        const Pre mp = prep_record(a, mine);
        Texel T = load_texel(a, t);
        for (uint32_t i = 0; i < k; ++i) {
            Pre q;
            q.key = __shfl_sync(FULL, mp.key, i);
            q.mode = __shfl_sync(FULL, mp.mode, i);
            q.d1 = __shfl_sync(FULL, mp.d1, i);
            q.d0 = __shfl_sync(FULL, mp.d0, i);
            q.s1n = __shfl_sync(FULL, mp.s1n, i);
            q.s0n = __shfl_sync(FULL, mp.s0n, i);
            q.wi = __shfl_sync(FULL, mp.wi, i);
            q.mzi = __shfl_sync(FULL, mp.mzi, i);
            q.mwi = __shfl_sync(FULL, mp.mwi, i);
            RecOut o;
            if (!apply_prepared(q, T, o)) {  // uniform: every lane holds the same texel state
                Rec r;
                r.key = q.key;
                r.multipl = __shfl_sync(FULL, mine.multipl, i);
                r.sc = __shfl_sync(FULL, mine.sc, i);
                r.vol = __shfl_sync(FULL, mine.vol, i);
                r.s0 = __shfl_sync(FULL, mine.s0, i);
                r.s1 = __shfl_sync(FULL, mine.s1, i);
                r.vx = __shfl_sync(FULL, mine.vx, i);
                r.vy = __shfl_sync(FULL, mine.vy, i);
                r.kill = __shfl_sync(FULL, mine.kill, i);
                o = apply_record(a, r, T);
            }
            if ((uint32_t)lane == i) store_rec(a, q.key, o);
        }
        if (lane == 0) store_texel(a, t, T);
    }
}

// one warp per big texel (more than 32 records): sort the bucket by droplet
// id (bitonic network in shared memory, chunks of HOT_KEYS merged by rank),
// then stage 32 prepared records at a time in shared memory for lane 0's
// sequential update
__global__ void __launch_bounds__(32 * HOT_WARPS) k_papply_big(const ApplyArgs a) {
    __shared__ uint32_t sk[HOT_WARPS][HOT_KEYS];
    __shared__ Rec sr[HOT_WARPS][32];
    __shared__ Pre sp[HOT_WARPS][32];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const uint32_t nbig = min(a.hot[1], a.hot_cap);
    for (uint32_t h = blockIdx.x * HOT_WARPS + wl; h < nbig; h += gridDim.x * HOT_WARPS) {
        const size_t t = a.hot[2 + a.hot_cap + h];
        const uint32_t lo = a.offs[t], hi = a.offs[t + 1], k = hi - lo;
        // sort chunks of up to HOT_KEYS records in shared memory into
        // `sorted`; a bucket of several chunks is then merged into `keys` by
        // each record's rank (its place in its chunk plus, per other chunk,
        // the records below it found by binary search)
        for (uint32_t c0 = 0; c0 < k; c0 += HOT_KEYS) {
            const uint32_t len = min((uint32_t)HOT_KEYS, k - c0);
            uint32_t P = 32;
            while (P < len) P <<= 1;
            for (uint32_t i = lane; i < P; i += 32) sk[wl][i] = i < len ? a.keys[lo + c0 + i] : 0xffffffffu;
            __syncwarp();
            for (uint32_t size = 2; size <= P; size <<= 1)
                for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
                    for (uint32_t q = lane; q < P / 2; q += 32) {
                        const uint32_t pos = 2 * stride * (q / stride) + (q % stride), par = pos + stride;
                        const bool up = (pos & size) == 0;
                        const uint32_t u = sk[wl][pos], v = sk[wl][par];
                        if ((u > v) == up) {
                            sk[wl][pos] = v;
                            sk[wl][par] = u;
                        }
                    }
                    __syncwarp();
                }
            for (uint32_t i = lane; i < len; i += 32) a.sorted[lo + c0 + i] = sk[wl][i];
            __syncwarp();
        }
        const bool merged = k > (uint32_t)HOT_KEYS;
        if (merged) {
            for (uint32_t i = lane; i < k; i += 32) {
                const uint32_t key = a.sorted[lo + i];
                const uint32_t own = i / HOT_KEYS * HOT_KEYS;
                uint32_t rank = i - own;
                for (uint32_t c0 = 0; c0 < k; c0 += HOT_KEYS) {
                    if (c0 == own) continue;
                    uint32_t l = 0, h = min((uint32_t)HOT_KEYS, k - c0);  // records of chunk c0 below key
                    const uint32_t* ch = a.sorted + lo + c0;
                    while (l < h) {
                        const uint32_t m = (l + h) >> 1;
                        if (ch[m] < key) l = m + 1; else h = m;
                    }
                    rank += l;
                }
                a.keys[lo + rank] = key;
            }
        }
        const uint32_t* order = merged ? a.keys : a.sorted;
        __syncwarp();
        Texel T = load_texel(a, t);
        for (uint32_t base = lo; base < hi; base += 32) {
            const uint32_t m = min(32u, hi - base);
            if ((uint32_t)lane < m) {
                const Rec r = load_rec(a, order[base + lane]);
                sr[wl][lane] = r;
                sp[wl][lane] = prep_record(a, r);
            }
            __syncwarp();
            if (lane == 0)
                for (uint32_t i = 0; i < m; ++i) {
                    RecOut o;
                    if (!apply_prepared(sp[wl][i], T, o)) o = apply_record(a, sr[wl][i], T);
                    store_rec(a, sp[wl][i].key, o);
                }
            __syncwarp();
        }
        if (lane == 0) store_texel(a, t, T);
    }
}

// each droplet replays its corners 0..3 for its sediment
__global__ void k_pfinal(const hg_erosion_settings es, Drops d, int n, const float* __restrict__ rec,
                         const uint8_t* __restrict__ rec_mask) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= d.count || d.iters[id] == 0) return;
    const float old_sed[2] = {d.s0[id], d.s1[id]};
    float sed[2] = {old_sed[0], old_sed[1]};
    const bool kill = d.kill[id] != 0;
    for (int k = 0; k < 4; ++k) {
        int cx, cy;
        float multipl;
        corner(d.px[id], d.py[id], k, n, cx, cy, multipl);
        const uint32_t key = (uint32_t)id * 4u + (uint32_t)k;
        if (kill) {
            sed[1] -= old_sed[1] * multipl;
            sed[0] -= old_sed[0] * multipl;
        } else {
            const uint32_t m = rec_mask[key];
            if (m & 2u) sed[1] = rec[2 * key + 0];
            if (m & 1u) sed[0] = rec[2 * key + 1];
        }
        const float conv = sed[0] * es.Kconv * es.d_t;
        sed[1] += conv;
        sed[0] -= conv;
    }
    d.s0[id] = sed[0];
    d.s1[id] = sed[1];
}

struct SmoothArgs {
    float m;       // clamp(Kspeed[1] * d_t, 0, 1)
    float count;   // droplets
    int n;
    const float* rock;
    const float* dirt;
    const float* water;
    float* rock_o;
    float* dirt_o;
    float* water_o;
    const float* mom[4];
    float* mom_o[4];
};

// glsl/smoothing.glsl:22-103 with the particle branch (:76-95); border texels
// copy their height and leave the momentum map's write buffer untouched
__global__ void k_psmooth(const SmoothArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = a.n;
    if (x >= n || y >= n) return;
    const size_t i = (size_t)y * n + x;
    float r = a.rock[i], g = a.dirt[i], wat = a.water[i];
    if (x == 0 || y == 0 || x == n - 1 || y == n - 1) {
        a.rock_o[i] = r;
        a.dirt_o[i] = g;
        a.water_o[i] = wat;
        return;
    }
    cell_smooth2(a.m, r, g, a.rock[i - 1], a.dirt[i - 1], a.rock[i + 1], a.dirt[i + 1], a.rock[i + n], a.dirt[i + n],
                 a.rock[i - n], a.dirt[i - n]);
    float mx = a.mom[0][i], my = a.mom[1][i], mz = a.mom[2][i], mw = a.mom[3][i];
    const float keep = gclamp(1.0f - 1e-12f * a.count, 0.0f, 1.0f);
    mx *= keep;
    my *= keep;
    mx += 1e-12f * a.count * mz;
    my += 1e-12f * a.count * mw;
    mz = 0.0f;
    mw = 0.0f;
    wat *= gclamp(1.0f - 8e-8f * a.count, 0.0f, 1.0f);
    if (wat < 1e-6f) wat = 0.0f;
    if (sqrtf(mx * mx + my * my) < 1e-12f) { mx = 0.0f; my = 0.0f; }
    a.mom_o[0][i] = mx; a.mom_o[1][i] = my; a.mom_o[2][i] = mz; a.mom_o[3][i] = mw;
    a.rock_o[i] = r;
    a.dirt_o[i] = g;
    a.water_o[i] = wat;
}

}  // namespace

size_t particle_scan_blocks(size_t cells) { return (cells + SCAN_T * SCAN_E - 1) / (SCAN_T * SCAN_E); }
size_t particle_hot_capacity(size_t cells, int count) {
    return std::min(cells, (size_t)4 * (size_t)count / (SMALL + 1) + 1);
}

void launch_particle_step(const StepConsts& c, const hg_erosion_settings& es, const ParticleBufs& pb,
                          const PWorld& pw, uint32_t step1, uint64_t seed, bool should_rain, cudaStream_t st) {
    const int n = c.n;
    const size_t cells = (size_t)n * n;
    const int pgrid = (pb.d.count + PB - 1) / PB;
    MoveArgs ma{c, es, pb.d, pw.rock, pw.dirt, pw.water, pw.mom[0], pw.mom[1], step1, (uint32_t)seed,
                (uint32_t)(seed >> 32), should_rain ? 1 : 0};
    k_pmove<<<pgrid, PB, 0, st>>>(ma);
    cudaMemsetAsync(pb.cnt, 0, cells * sizeof(uint32_t), st);
    k_pcount<<<pgrid, PB, 0, st>>>(pb.d, n, pb.cnt);
    const size_t nb = particle_scan_blocks(cells);
    k_scan_blocks<<<(unsigned)nb, SCAN_T, 0, st>>>(pb.cnt, pb.offs, cells, pb.block_sums);
    k_scan_sums<<<1, SCAN_T, 0, st>>>(pb.block_sums, (int)nb, pb.offs + cells);
    k_scan_add<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(pb.offs, pb.cursor, cells, pb.block_sums);
    k_pscatter<<<pgrid, PB, 0, st>>>(pb.d, n, pb.cursor, pb.keys);
    ApplyArgs aa{es, pb.d, n, pb.offs, pb.keys, pb.sorted, pb.hot, pb.hot_cap, pw.rock, pw.dirt, pw.water,
                 pw.mom[2], pw.mom[3], pb.rec, pb.rec_mask};
    cudaMemsetAsync(pb.hot, 0, 2 * sizeof(uint32_t), st);
    dim3 g((n + BX - 1) / BX, (n + BY - 1) / BY);
    k_papply<<<g, dim3(BX, BY), 0, st>>>(aa);
    k_papply_mid<<<152 * 12, 32 * HOT_WARPS, 0, st>>>(aa);
    k_papply_big<<<152 * 4, 32 * HOT_WARPS, 0, st>>>(aa);
    k_pfinal<<<pgrid, PB, 0, st>>>(es, pb.d, n, pb.rec, pb.rec_mask);
    count_launch(10);
}

void launch_particle_smooth(const StepConsts& c, float count, const PWorld& in, const PWorld& out, cudaStream_t st) {
    SmoothArgs sa;
    sa.m = c.smooth_m;
    sa.count = count;
    sa.n = c.n;
    sa.rock = in.rock; sa.dirt = in.dirt; sa.water = in.water;
    sa.rock_o = out.rock; sa.dirt_o = out.dirt; sa.water_o = out.water;
    for (int k = 0; k < 4; ++k) {
        sa.mom[k] = in.mom[k];
        sa.mom_o[k] = out.mom[k];
    }
    dim3 g((c.n + BX - 1) / BX, (c.n + BY - 1) / BY);
    k_psmooth<<<g, dim3(BX, BY), 0, st>>>(sa);
    count_launch();
}

}  // namespace hg
