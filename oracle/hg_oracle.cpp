// hydro-gen grid-erosion ORACLE — test infrastructure only.
//
// A CPU restatement of hydro-gen's GLSL grid-erosion passes, templated on the
// arithmetic type (float = the reference's own precision, double = the
// accuracy reference).  It keeps the reference's data layout: every field is
// an RGBA texture (4 channels per cell, row-major, x fastest) and every pass
// reads the "read" texture of a ping-pong pair and writes the "write" one,
// exactly as gl::Tex_pair does (src/shaderprogram.cpp:51-72).
//
// Only tests, the smoke check and the CPU-baseline legs of the benchmark load
// this library; the product library never links or calls it.
//
// Parity unpinned: hydro-gen ships no tests, golden vectors or fixtures, and
// its passes are GLSL that only an OpenGL 4.6 driver can run (no graphics
// stack exists on these machines).  The restatement is pinned instead by
// hand-derived known-answer cases with closed-form outcomes
// (tests/test_oracle_kat.py) and by line-by-line citations below.
//
// Reference sources followed (paths inside the hydro-gen project):
//   rain pass .................. glsl/rain.glsl:32-56 (the amount model is the
//                                uniform / Bernoulli rain of the benchmark
//                                workloads, see rain_pass)
//   hydro_flux ................. glsl/hydro_flux.glsl:33-47, 77-166
//   hydro_erosion .............. glsl/hydro_erosion.glsl:23-92
//   sediment_transport ......... glsl/sediment_transport.glsl:26-30, 66-93
//   img_bilinear ............... glsl/img_interpolation.glsl:3-22
//   thermal_erosion ............ glsl/thermal_erosion.glsl:20-115
//   thermal_transport .......... glsl/thermal_transport.glsl:15-65
//   smoothing .................. glsl/smoothing.glsl:22-103 (grid branch)
//   step sequencing ............ src/erosion.cpp:103-121, 158-200,
//                                rain cadence src/main.cpp:315-320
//   settings layout ............ glsl/bindings.glsl:39-60
//
// GLSL semantics made explicit: min(x,y) = y<x?y:x, max(x,y) = x<y?y:x,
// clamp = min(max(x,lo),hi), mix(x,y,a) = x*(1-a)+y*a, fract(x) = x-floor(x),
// smoothstep by its formula (also for edge0 > edge1), length = sqrt(dot),
// normalize = v / length(v), int(float) truncates, out-of-range texelFetch /
// imageLoad return 0, expressions evaluate left to right with one rounding per
// operation (no fused multiply-add: build with -ffp-contract=off).
//
// GLSL leaves atan's precision to the driver.  The float instantiation uses
// the library's polynomial arctangent (coefficients from
// oracle/fit_atan.py, restated here) so that float results can
// be compared bit for bit; the double instantiation uses std::atan.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstddef>
#include <vector>
#include <type_traits>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// Mirror of Erosion_data (glsl/bindings.glsl:39-60), std140 layout, 96 bytes.
struct OracleErosion {
    uint32_t particle_count;   // 0
    float Kc;                  // 4
    float Kalpha[2];           // 8
    float Kconv;               // 16
    float pad0;                // 20
    float Ks[2];               // 24
    float Kd[2];               // 32
    float Ke;                  // 40
    float ENERGY_KEPT;         // 44
    float Kspeed[2];           // 48
    float G;                   // 56
    float d_t;                 // 60
    float density, init_volume, friction, inertia, min_volume, min_velocity; // 64..84
    uint32_t ttl;              // 88
    uint32_t pad1;             // 92
};

// Rain model and pass switches used by the benchmark workloads.
struct OracleOptions {
    int32_t rain_mode;         // 0 off, 1 uniform, 2 Bernoulli (Philox4x32-10)
    int32_t rain_period;       // rain on step n (1-based) when n % period == 0
    float rain_amount;         // water added per raining cell
    uint32_t rain_threshold;   // Bernoulli: rain when philox word < threshold
    uint64_t rain_seed;        // Philox key
    uint32_t terrain_id;       // fourth Philox counter word
    int32_t skip_identity;     // skip thermal layers with Kspeed==0 and the
                               // smoothing pass when Kspeed[1]==0 (exact)
    // rain_mode 3: the reference's rain (glsl/rain.glsl:32-56, hg_terrain_ref.cpp)
    float rain_time0, rain_time_step;  // frame time of step n: time0 + n * time_step
    float mountain_thresh, mountain_multip, drops, max_height;
};

// glsl/rain.glsl's increment of one cell (hg_terrain_ref.cpp)
float hgo_ref_rain_cell(int x, int y, float total, float time, float amount, float mountain_thresh,
                        float mountain_multip, float drops, float max_height);

}  // extern "C"

static_assert(sizeof(OracleErosion) == 96, "Erosion_data is 96 bytes");
static_assert(offsetof(OracleErosion, Ks) == 24, "std140 offset of Ks");
static_assert(offsetof(OracleErosion, d_t) == 60, "std140 offset of d_t");

namespace {

template <typename T> struct V4 {
    T x = 0, y = 0, z = 0, w = 0;
    T& operator[](int i) { return i == 0 ? x : i == 1 ? y : i == 2 ? z : w; }
    T operator[](int i) const { return i == 0 ? x : i == 1 ? y : i == 2 ? z : w; }
};

// ---- GLSL built-ins --------------------------------------------------------
template <typename T> inline T gmin(T x, T y) { return y < x ? y : x; }
template <typename T> inline T gmax(T x, T y) { return x < y ? y : x; }
template <typename T> inline T gclamp(T x, T lo, T hi) { return gmin(gmax(x, lo), hi); }
template <typename T> inline T gmix(T x, T y, T a) { return x * (T(1) - a) + y * a; }
template <typename T> inline T gfract(T x) { return x - std::floor(x); }
template <typename T> inline T gsmoothstep(T e0, T e1, T x) {
    T t = gclamp((x - e0) / (e1 - e0), T(0), T(1));
    return t * t * (T(3) - T(2) * t);
}
template <typename T> inline T glength2(T x, T y) { return std::sqrt(x * x + y * y); }

// Polynomial arctangent (float), see the header comment.
// u + u*(s*P(s)), s = u*u, for |u| <= tan(pi/8)
inline float poly_atan_core(float u) {
    const float c0 = -3.333333135e-01f, c1 = 1.999990344e-01f, c2 = -1.428200752e-01f,
                c3 = 1.104469076e-01f, c4 = -8.476266265e-02f, c5 = 4.744043201e-02f;
    float s = u * u;
    float p = c5;
    p = p * s; p = p + c4;
    p = p * s; p = p + c3;
    p = p * s; p = p + c2;
    p = p * s; p = p + c1;
    p = p * s; p = p + c0;
    float q = s * p;
    q = u * q;
    return u + q;
}
inline float poly_atanf(float x) {
    float ax = std::fabs(x), r;
    if (ax <= 0.414213562f) r = poly_atan_core(ax);
    else if (ax <= 2.41421356f) r = 0.785398163f + poly_atan_core((ax - 1.0f) / (ax + 1.0f));
    else r = 1.57079637f - poly_atan_core(1.0f / ax);
    return std::copysign(r, x);
}
// The float instantiation's arctangent: 0 = poly_atanf (the kernels' own,
// for bit parity), 1 = the C library's atanf.  The second exists only to
// measure how far the choice of arctangent moves the float result from FP64.
static int g_float_atan_libm = 0;
inline float o_atan(float x) { return g_float_atan_libm ? std::atan(x) : poly_atanf(x); }
// Depth below which the flux pass sets the velocity to 0 (both
// instantiations); 0 (the default) is the reference's scheme.  Exists only to
// measure how much of the float-vs-FP64 distance the velocity of thin water
// films (old-flux difference / depth) accounts for.
static double g_film_guard = 0.0;
inline double o_atan(double x) { return std::atan(x); }

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) ---------------------
inline void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}
inline void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c0, hi0, lo0);
        mulhilo32(0xCD9E8D57u, c2, hi1, lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
// One Philox call covers four horizontally adjacent cells:
// counter = (x/4, y, step, terrain_id), key = seed; cell x uses word x%4.
inline uint32_t rain_word(int x, int y, uint64_t step, uint32_t terrain, uint64_t seed) {
    uint32_t ctr[4] = {(uint32_t)x >> 2, (uint32_t)y, (uint32_t)step, terrain};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t out[4];
    philox4x32_10(ctr, key, out);
    return out[x & 3];
}

// ---- world -----------------------------------------------------------------
template <typename T> struct Pair {
    std::vector<V4<T>> tex[2];
    int r = 0;  // index of the read texture
    const std::vector<V4<T>>& rd() const { return tex[r]; }
    std::vector<V4<T>>& wr() { return tex[1 - r]; }
    void swap() { r = 1 - r; }
    void init(size_t n) { tex[0].assign(n, V4<T>{}); tex[1].assign(n, V4<T>{}); r = 0; }
};

template <typename T> struct World {
    int n = 0;
    uint64_t step = 0;   // completed steps
    Pair<T> height;      // (rock, dirt, water, total)
    Pair<T> flux;        // (fL, fR, fT, fB)
    Pair<T> vel;         // (u, v, d1+d2, unused)
    Pair<T> sed;         // (s_rock, s_dirt, 0, 0)
    Pair<T> thc;         // thermal cross outflow (L, R, T, B)
    Pair<T> thd;         // thermal diagonal outflow (LT, RT, LB, RB)
    std::vector<float> ks;  // optional per-cell rock solubility (replaces Ks[0])
    // particle mode (glsl/particle.glsl): Particle (glsl/bindings.glsl:101-110)
    struct Drop {
        float sc = 0;
        uint32_t iters = 0;
        float px = 0, py = 0, vx = 0, vy = 0, vol = 0;
        float sed[2] = {0, 0};
        bool kill = false;
    };
    std::vector<Drop> drops;
    World(int n_) : n(n_) {
        size_t c = (size_t)n * n;
        height.init(c); flux.init(c); vel.init(c); sed.init(c); thc.init(c); thd.init(c);
    }
    size_t id(int x, int y) const { return (size_t)y * n + x; }
    bool inb(int x, int y) const { return x >= 0 && x < n && y >= 0 && y < n; }
    // rows the grid passes compute ([row_lo, row_end()); all by default): a
    // slab of a row decomposition computes only its own rows, its halo rows
    // are copied in between passes
    int row_lo = 0, row_hi = -1;
    int row_end() const { return row_hi < 0 ? n : row_hi; }
};

#define OMP_ROWS _Pragma("omp parallel for schedule(static)")

// frame time of step n for the reference rain (computed in double, as the
// library's host does, then rounded to float)
inline float rain_time(const OracleOptions& o, uint64_t n) {
    return (float)((double)o.rain_time0 + (double)n * (double)o.rain_time_step);
}

// glsl/rain.glsl:32-56 (the water increment follows the workload's rain model)
template <typename T> void rain_pass(World<T>& w, const OracleOptions& o, uint64_t step_1based) {
    const auto& src = w.height.rd();
    auto& dst = w.height.wr();
    const T amount = T(o.rain_amount);
    OMP_ROWS
    for (int y = w.row_lo; y < w.row_end(); ++y)
        for (int x = 0; x < w.n; ++x) {
            V4<T> terr = src[w.id(x, y)];
            T incr = T(0);
            if (o.rain_mode == 1) incr = amount;
            else if (o.rain_mode == 3)
                incr = T(hgo_ref_rain_cell(x, y, (float)terr.w, rain_time(o, step_1based), o.rain_amount,
                                           o.mountain_thresh, o.mountain_multip, o.drops, o.max_height));
            else if (rain_word(x, y, step_1based, o.terrain_id, o.rain_seed) < o.rain_threshold) incr = amount;
            terr.z += incr;
            terr.w = terr.x + terr.y + terr.z;
            dst[w.id(x, y)] = terr;
        }
    w.height.swap();
}

// glsl/hydro_flux.glsl:77-166
template <typename T> void flux_pass(World<T>& w, const OracleErosion& s) {
    const auto& H = w.height.rd();
    const auto& F = w.flux.rd();
    const auto& VL = w.vel.rd();
    auto& Ho = w.height.wr();
    auto& Fo = w.flux.wr();
    auto& Vo = w.vel.wr();
    const T EK = T(s.ENERGY_KEPT), dt = T(s.d_t), G = T(s.G), A = T(1), L = T(1);
    const T FAR = T(999999999999.0);
    const int n = w.n;
    OMP_ROWS
    for (int y = w.row_lo; y < w.row_end(); ++y)
        for (int x = 0; x < n; ++x) {
            auto wh = [&](int xx, int yy) -> T { return w.inb(xx, yy) ? H[w.id(xx, yy)].w : FAR; };
            auto gf = [&](int xx, int yy) -> V4<T> { return w.inb(xx, yy) ? F[w.id(xx, yy)] : V4<T>{}; };
            V4<T> out = gf(x, y);
            V4<T> vel = VL[w.id(x, y)];
            V4<T> terrain = H[w.id(x, y)];
            T d1 = terrain.z;
            V4<T> dh;
            dh.x = terrain.w - wh(x - 1, y);
            dh.y = terrain.w - wh(x + 1, y);
            dh.z = terrain.w - wh(x, y + 1);
            dh.w = terrain.w - wh(x, y - 1);
            V4<T> in;
            in.x = gf(x - 1, y).y;
            in.y = gf(x + 1, y).x;
            in.z = gf(x, y + 1).w;
            in.w = gf(x, y - 1).z;
            out.x = gmax(T(0), EK * out.x + dt * A * (G * dh.x) / L);
            out.y = gmax(T(0), EK * out.y + dt * A * (G * dh.y) / L);
            out.z = gmax(T(0), EK * out.z + dt * A * (G * dh.z) / L);
            out.w = gmax(T(0), EK * out.w + dt * A * (G * dh.w) / L);
            if (x <= 0) out.x = 0;
            else if (x >= n - 1) out.y = 0;
            if (y <= 0) out.w = 0;
            else if (y >= n - 1) out.z = 0;
            T sum_in = in.x + in.y + in.z + in.w;
            T sum_out = out.x + out.y + out.z + out.w;
            T K = gmin(T(1), (terrain.z * L * L) / (sum_out * dt));
            out.x *= K; out.y *= K; out.z *= K; out.w *= K;
            sum_out *= K;
            T d_volume = dt * (sum_in - sum_out);
            T d2 = gmax(T(0), d1 + (d_volume / (L * L)));
            terrain.z = d2;
            terrain.w = terrain.x + d2 + terrain.y;
            vel.z = d1 + d2;
            if (vel.z > 0 && !(vel.z < T(g_film_guard))) {
                vel.x = (gf(x - 1, y).y - gf(x, y).x + gf(x, y).y - gf(x + 1, y).x) / (L * vel.z);
                vel.y = (gf(x, y - 1).z - gf(x, y).w + gf(x, y).z - gf(x, y + 1).w) / (L * vel.z);
            } else {
                vel.x = 0; vel.y = 0;
            }
            Fo[w.id(x, y)] = out;
            Vo[w.id(x, y)] = vel;
            Ho[w.id(x, y)] = terrain;
        }
    w.height.swap(); w.flux.swap(); w.vel.swap();
}

// glsl/hydro_erosion.glsl:23-92
template <typename T> void erosion_pass(World<T>& w, const OracleErosion& s) {
    const auto& H = w.height.rd();
    const auto& S = w.sed.rd();
    const auto& VL = w.vel.rd();
    auto& Ho = w.height.wr();
    auto& So = w.sed.wr();
    const T dt = T(s.d_t), Kc = T(s.Kc), Kconv = T(s.Kconv), L = T(1);
    const bool cell_ks = !w.ks.empty();
    const int n = w.n;
    OMP_ROWS
    for (int y = w.row_lo; y < w.row_end(); ++y)
        for (int x = 0; x < n; ++x) {
            auto ld = [&](int xx, int yy) -> V4<T> { return w.inb(xx, yy) ? H[w.id(xx, yy)] : V4<T>{}; };
            V4<T> vel = VL[w.id(x, y)];
            V4<T> terrain = H[w.id(x, y)];
            V4<T> sediment = S[w.id(x, y)];
            T dd = vel.z;
            T ero_vel = glength2(vel.x, vel.y);
            if (dd < T(1e-3)) {
                dd = gmax(T(5e-4), dd);
                ero_vel = gmix(glength2(vel.x, vel.y), T(0), gsmoothstep(T(1e-3), T(5e-4), dd));
            } else {
                ero_vel = glength2(vel.x, vel.y);
            }
            T cap = T(0);
            // get_terr_normal
            V4<T> r = ld(x + 1, y), l = ld(x - 1, y), b = ld(x, y - 1), t = ld(x, y + 1);
            T dx = r.x + r.y - l.x - l.y;
            T dz = t.x + t.y - b.x - b.y;
            // cross((2L, dx, 0), (0, dz, 2L))
            T ax = T(2) * L, ay = dx, az = T(0);
            T bx = T(0), by = dz, bz = T(2) * L;
            T cx = ay * bz - az * by;
            T cy = az * bx - ax * bz;
            T cz = ax * by - ay * bx;
            T len = std::sqrt(cx * cx + cy * cy + cz * cz);
            T ny = cy / len;
            T sin_a = std::fabs(std::sqrt(T(1) - ny * ny));
            for (int i = 1; i >= 0; --i) {
                T Ks_i = (i == 0 && cell_ks) ? T(w.ks[w.id(x, y)]) : T(s.Ks[i]);
                T Kls = dt * Ks_i;
                T Kld = dt * T(s.Kd[i]);
                T c = gmax(T(0), Kc * gmax(T(0.02), sin_a) * ero_vel - cap);
                if (c > sediment[i]) {
                    T old_terr = terrain[i];
                    terrain[i] -= Kls * (c - sediment[i]);
                    sediment[i] += Kls * (c - sediment[i]);
                    if (terrain[i] < 0) {
                        sediment[i] += terrain[i];
                        terrain[i] = 0;
                        cap += old_terr;
                    } else {
                        break;
                    }
                } else {
                    terrain[i] += Kld * (sediment[i] - c);
                    sediment[i] -= Kld * (sediment[i] - c);
                }
            }
            {
                T conv = sediment[0] * Kconv * dt;
                sediment[1] += conv;
                sediment[0] -= conv;
            }
            terrain.w = terrain.x + terrain.y + terrain.z;
            So[w.id(x, y)] = sediment;
            Ho[w.id(x, y)] = terrain;
        }
    w.height.swap(); w.sed.swap();
}

// glsl/img_interpolation.glsl:3-22 (out-of-range texels read as 0)
template <typename T> V4<T> bilinear(const World<T>& w, const std::vector<V4<T>>& img, T px, T py) {
    int ix = (int)px, iy = (int)py;  // ivec2(sample_pos): truncation
    T fx = gfract(px), fy = gfract(py);
    auto f = [&](int xx, int yy) -> V4<T> { return w.inb(xx, yy) ? img[w.id(xx, yy)] : V4<T>{}; };
    V4<T> a = f(ix, iy), b = f(ix + 1, iy), c = f(ix, iy + 1), d = f(ix + 1, iy + 1);
    V4<T> v1, v2, v;
    for (int k = 0; k < 4; ++k) {
        v1[k] = gmix(a[k], b[k], fx);
        v2[k] = gmix(c[k], d[k], fx);
        v[k] = gmix(v1[k], v2[k], fy);
    }
    return v;
}

// glsl/sediment_transport.glsl:26-30, 66-93
template <typename T> void sediment_pass(World<T>& w, const OracleErosion& s) {
    const auto& H = w.height.rd();
    const auto& S = w.sed.rd();
    const auto& VL = w.vel.rd();
    auto& Ho = w.height.wr();
    auto& So = w.sed.wr();
    const T dt = T(s.d_t), Ke = T(s.Ke);
    const int n = w.n;
    const T maxc = T(n - 1);
    OMP_ROWS
    for (int y = w.row_lo; y < w.row_end(); ++y)
        for (int x = 0; x < n; ++x) {
            V4<T> vel = VL[w.id(x, y)];
            T bx = T(x) - vel.x * dt;
            T by = T(y) - vel.y * dt;
            bx = gclamp(bx, T(0), maxc);
            by = gclamp(by, T(0), maxc);
            V4<T> st = bilinear(w, S, bx, by);
            V4<T> terrain = H[w.id(x, y)];
            terrain.z *= (T(1) - Ke * dt);
            terrain.w = terrain.x + terrain.y + terrain.z;
            So[w.id(x, y)] = st;
            Ho[w.id(x, y)] = terrain;
        }
    w.height.swap(); w.sed.swap();
}

// glsl/thermal_erosion.glsl:20-115
template <typename T> void thermal_flux_pass(World<T>& w, const OracleErosion& s, int layer) {
    const auto& H = w.height.rd();
    auto& Co = w.thc.wr();
    auto& Do = w.thd.wr();
    const T dt = T(s.d_t), a = T(1), L = T(1), WS = T(1);
    const T FAR = T(999999999999.0);
    const T Kl_alph = T(s.Kalpha[layer]);
    const T Klspeed = T(s.Kspeed[layer]);
    const int n = w.n;
    const int ox[2][4] = {{-1, 1, 0, 0}, {-1, 1, -1, 1}};
    const int oy[2][4] = {{0, 0, 1, -1}, {1, 1, -1, -1}};
    OMP_ROWS
    for (int y = w.row_lo; y < w.row_end(); ++y)
        for (int x = 0; x < n; ++x) {
            auto gh = [&](int xx, int yy) -> V4<T> {
                if (!w.inb(xx, yy)) return V4<T>{FAR, FAR, FAR, FAR};
                return H[w.id(xx, yy)];
            };
            V4<T> terrain = H[w.id(x, y)];
            V4<T> d_h[2];
            for (int i = 0; i <= layer; ++i)
                for (int j = 0; j < 2; ++j)
                    for (int k = 0; k < 4; ++k)
                        d_h[j][k] += terrain[i] - gh(x + ox[j][k], y + oy[j][k])[i];
            T Hh = 0;
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 4; ++k)
                    if (d_h[j][k] > Hh) Hh = d_h[j][k];
            Hh = gmin(terrain[layer], Hh);
            V4<T> out[2];
            T bk = 0;
            T sharpness = 1;
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 4; ++k) {
                    T b = d_h[j][k];
                    if (b <= 0) { out[j][k] = 0; continue; }
                    T d = L;
                    if (j == 1) d *= std::sqrt(T(2));
                    T alph = o_atan(b / (d / WS));
                    if (alph > Kl_alph) {
                        T newsh = T(1) + alph - Kl_alph;
                        if (newsh > sharpness) sharpness = newsh;
                        bk += b;
                        out[j][k] = 1;
                        continue;
                    }
                    out[j][k] = 0;
                }
            sharpness *= sharpness * sharpness;
            T S = dt * Klspeed * sharpness * a * Hh / T(2);
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 4; ++k)
                    out[j][k] = (out[j][k] == 1) ? S * d_h[j][k] / bk : T(0);
            Co[w.id(x, y)] = out[0];
            Do[w.id(x, y)] = out[1];
        }
    w.thc.swap(); w.thd.swap();
}

// glsl/thermal_transport.glsl:15-65
template <typename T> void thermal_transport_pass(World<T>& w, int layer) {
    const auto& H = w.height.rd();
    const auto& C = w.thc.rd();
    const auto& D = w.thd.rd();
    auto& Ho = w.height.wr();
    const int n = w.n;
    OMP_ROWS
    for (int y = w.row_lo; y < w.row_end(); ++y)
        for (int x = 0; x < n; ++x) {
            auto g = [&](const std::vector<V4<T>>& img, int xx, int yy) -> V4<T> {
                return w.inb(xx, yy) ? img[w.id(xx, yy)] : V4<T>{};
            };
            V4<T> terrain = H[w.id(x, y)];
            T in_flux = 0;
            in_flux += g(C, x - 1, y).y;
            in_flux += g(C, x + 1, y).x;
            in_flux += g(C, x, y + 1).w;
            in_flux += g(C, x, y - 1).z;
            in_flux += g(D, x - 1, y + 1).w;
            in_flux += g(D, x + 1, y + 1).z;
            in_flux += g(D, x - 1, y - 1).y;
            in_flux += g(D, x + 1, y - 1).x;
            T sum_flux = 0;
            V4<T> o0 = C[w.id(x, y)], o1 = D[w.id(x, y)];
            for (int k = 0; k < 4; ++k) sum_flux -= o0[k];
            for (int k = 0; k < 4; ++k) sum_flux -= o1[k];
            sum_flux += in_flux;
            terrain[layer] += sum_flux;
            terrain.w = terrain.x + terrain.y + terrain.z;
            Ho[w.id(x, y)] = terrain;
        }
    w.height.swap();
}

// glsl/smoothing.glsl:22-103, grid branch (particle_count == 0)
template <typename T> void smoothing_pass(World<T>& w, const OracleErosion& s) {
    const auto& H = w.height.rd();
    auto& Ho = w.height.wr();
    const T d_time = T(s.d_t);
    const int n = w.n;
    OMP_ROWS
    for (int y = w.row_lo; y < w.row_end(); ++y)
        for (int x = 0; x < n; ++x) {
            V4<T> terrain = H[w.id(x, y)];
            T tr = terrain.x, tg = terrain.y;
            if (x == 0 || y == 0 || x == n - 1 || y == n - 1) {
                Ho[w.id(x, y)] = terrain;
                continue;
            }
            V4<T> L4 = H[w.id(x - 1, y)], R4 = H[w.id(x + 1, y)], T4 = H[w.id(x, y + 1)], B4 = H[w.id(x, y - 1)];
            T lr = L4.x, lg = L4.y, rr = R4.x, rg = R4.y, trr = T4.x, tgg = T4.y, br = B4.x, bg = B4.y;
            T dlr = tr - lr, dlg = tg - lg; dlg += dlr;
            T drr = tr - rr, drg = tg - rg; drg += drr;
            T dtr = tr - trr, dtg = tg - tgg; dtg += dtr;
            T dbr = tr - br, dbg = tg - bg; dbg += dbr;
            T g_hdiff = (dlg + drg + dtg + dbg) / T(4);
            T r_hdiff = (dlr + drr + dtr + dbr) / T(4);
            g_hdiff = std::fabs(g_hdiff);
            r_hdiff = std::fabs(r_hdiff);
            T xr = dlr * drr, xg = dlg * drg;
            T yr = dtr * dbr, yg = dtg * dbg;
            T nr = tr, ng = tg;
            if ((((-dlr) > r_hdiff || (-drr) > r_hdiff) && xr > 0) ||
                (((-dtr) > r_hdiff || (-dbr) > r_hdiff) && yr > 0))
                nr = (tr + lr + rr + trr + br) / T(5);
            if ((((-dlg) > g_hdiff || (-drg) > g_hdiff) && xg > 0) ||
                (((-dtg) > g_hdiff || (-dbg) > g_hdiff) && yg > 0))
                ng = (tg + lg + rg + tgg + bg) / T(5);
            T multip = gclamp(T(s.Kspeed[1]) * d_time, T(0), T(1));
            terrain.x = multip * nr + (T(1) - multip) * terrain.x;
            terrain.y = multip * ng + (T(1) - multip) * terrain.y;
            terrain.w = terrain.x + terrain.y + terrain.z;
            Ho[w.id(x, y)] = terrain;
        }
    w.height.swap();
}

// src/erosion.cpp:158-200 + src/main.cpp:315-320
template <typename T> void one_step(World<T>& w, const OracleErosion& s, const OracleOptions& o) {
    uint64_t n1 = w.step + 1;  // the reference increments the counter before the rain test
    if (o.rain_mode != 0 && o.rain_period > 0 && (n1 % (uint64_t)o.rain_period) == 0) rain_pass(w, o, n1);
    flux_pass(w, s);
    erosion_pass(w, s);
    sediment_pass(w, s);
    for (int layer = 0; layer < 2; ++layer) {
        if (o.skip_identity && s.Kspeed[layer] == 0.0f) continue;
        thermal_flux_pass(w, s, layer);
        thermal_transport_pass(w, layer);
    }
    if (!(o.skip_identity && s.Kspeed[1] == 0.0f)) smoothing_pass(w, s);
    w.step = n1;
}

// ---- particle mode: src/erosion.cpp:132-156 ------------------------------------
// The reference spawns droplets at fract(1e4 sin(...))-hashed positions keyed
// by the frame time; no two libms agree on those sines, so spawn positions
// here come from Philox4x32-10 with counter (particle id, step, 'part', 0)
// and the rain seed as key, a 24-bit uniform per axis.
inline float spawn_uniform(uint32_t word) { return (float)(word >> 8) * 0x1p-24f; }

// img_bilinear (glsl/img_interpolation.glsl:3-22) of one channel, 0 outside
inline float bilin(const World<float>& w, const std::vector<V4<float>>& img, int ch, float sx, float sy) {
    int ix = (int)sx, iy = (int)sy;
    float fx = gfract(sx), fy = gfract(sy);
    auto f = [&](int xx, int yy) -> float { return w.inb(xx, yy) ? img[w.id(xx, yy)][ch] : 0.0f; };
    float v1 = gmix(f(ix, iy), f(ix + 1, iy), fx);
    float v2 = gmix(f(ix, iy + 1), f(ix + 1, iy + 1), fx);
    return gmix(v1, v2, fy);
}

// glsl/particle.glsl:64-136
void particle_move_pass(World<float>& w, const OracleErosion& s, bool should_rain, uint64_t step1, uint64_t seed) {
    const auto& H = w.height.rd();
    const auto& M = w.vel.rd();
    const float dt = s.d_t;
    const float span = (float)w.n - 4.0f;
    for (size_t id = 0; id < w.drops.size(); ++id) {
        auto p = w.drops[id];
        if (p.iters == 0 && !should_rain) continue;
        for (int i = 0; i < 2; ++i)
            if (p.sed[i] < 0.0f || p.iters == 0) p.sed[i] = 0.0f;
        if (p.iters == 0 || p.kill) {
            uint32_t ctr[4] = {(uint32_t)id, (uint32_t)step1, 0x70617274u, 0u};
            uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
            uint32_t out[4];
            philox4x32_10(ctr, key, out);
            p.kill = false;
            p.px = spawn_uniform(out[0]) * span / 1.0f + 2.0f;
            p.py = spawn_uniform(out[1]) * span / 1.0f + 2.0f;
            p.vx = 0.0f;
            p.vy = 0.0f;
            p.vol = s.init_volume;
            p.iters = should_rain ? 1u : 0u;
            if (!should_rain) { w.drops[id] = p; continue; }
        }
        // get_terr_normal (:48-60)
        float rr = bilin(w, H, 0, p.px + 1.0f, p.py), rg = bilin(w, H, 1, p.px + 1.0f, p.py);
        float lr = bilin(w, H, 0, p.px - 1.0f, p.py), lg = bilin(w, H, 1, p.px - 1.0f, p.py);
        float br = bilin(w, H, 0, p.px, p.py - 1.0f), bg = bilin(w, H, 1, p.px, p.py - 1.0f);
        float tr = bilin(w, H, 0, p.px, p.py + 1.0f), tg = bilin(w, H, 1, p.px, p.py + 1.0f);
        float dx = rr + rg - lr - lg;
        float dz = tr + tg - br - bg;
        float cx = dx * 2.0f - 0.0f * dz, cy = 0.0f * 0.0f - 2.0f * 2.0f, cz = 2.0f * dz - dx * 0.0f;
        float len = std::sqrt(cx * cx + cy * cy + cz * cz);
        float nx = cx / len, ny = cy / len, nz = cz / len;
        float mx = bilin(w, M, 0, p.px, p.py), my = bilin(w, M, 1, p.px, p.py);
        float water = bilin(w, H, 2, p.px, p.py);
        p.vx -= (dt * nx) / p.vol * s.G;
        p.vy -= (dt * nz) / p.vol * s.G;
        float lm = std::sqrt(mx * mx + my * my), lv = std::sqrt(p.vx * p.vx + p.vy * p.vy);
        if (lm > 0.0f && lv > 0.0f) {
            float d = (mx / lm) * (p.vx / lv) + (my / lm) * (p.vy / lv);
            float k = s.inertia * d / (p.vol + 1e5f * water);
            p.vx += k * mx;
            p.vy += k * my;
        }
        lv = std::sqrt(p.vx * p.vx + p.vy * p.vy);
        if (lv > 1.0f) { p.vx = p.vx / lv; p.vy = p.vy / lv; }
        float ox = p.px, oy = p.py;
        p.px += dt * p.vx;
        p.py += dt * p.vy;
        if (p.px <= 1.0f || p.py <= 1.0f || p.px * 1.0f >= (float)(w.n - 2) || p.py * 1.0f >= (float)(w.n - 2)) {
            p.px = ox; p.py = oy; p.vx = 0.0f; p.vy = 0.0f; p.kill = true;
        }
        float fr = 1.0f - dt * s.friction * ny;
        p.vx *= fr;
        p.vy *= fr;
        p.vol -= dt * s.Ke;
        float sin_a = std::fabs(std::sqrt(1.0f - ny * ny));
        lv = std::sqrt(p.vx * p.vx + p.vy * p.vy);
        p.sc = gmax(0.0f, s.Kc * p.vol * lv * gmax(0.02f, sin_a));
        p.iters++;
        if (p.vol <= s.min_volume || lv < s.min_velocity || p.iters >= s.ttl) p.kill = true;
        w.drops[id] = p;
    }
}

// glsl/particle_erosion.glsl:22-128, particles in id order, corners 0..3
void particle_erosion_pass(World<float>& w, const OracleErosion& s) {
    auto& H = w.height.tex[w.height.r];
    auto& M = w.vel.tex[w.vel.r];
    for (size_t id = 0; id < w.drops.size(); ++id) {
        if (w.drops[id].iters == 0) continue;
        const float px = w.drops[id].px, py = w.drops[id].py;
        const int bx = (int)(px * 1.0f), by = (int)(py * 1.0f);
        const float ofx = gfract(px * 1.0f), ofy = gfract(py * 1.0f);
        const int cxs[4] = {bx, bx + 1, bx + 1, bx}, cys[4] = {by, by, by + 1, by + 1};
        const float wx[4] = {1.0f - ofx, ofx, ofx, 1.0f - ofx}, wy[4] = {1.0f - ofy, 1.0f - ofy, ofy, ofy};
        const float old_sed[2] = {w.drops[id].sed[0], w.drops[id].sed[1]};
        for (int k = 0; k < 4; ++k) {
            auto part = w.drops[id];
            V4<float> terr = H[w.id(cxs[k], cys[k])];
            V4<float> mom = M[w.id(cxs[k], cys[k])];
            const float multipl = wx[k] * wy[k];
            float cap = 0.0f;
            for (int i = 1; i >= 0; --i) {
                if (part.kill) {
                    float sed = old_sed[i] * multipl;
                    terr[i] += sed;
                    part.sed[i] -= sed;
                    continue;
                }
                const float Kls = s.d_t * s.Ks[i], Kld = s.d_t * s.Kd[i];
                const float c = gmax(0.0f, part.sc - cap);
                float s1 = old_sed[i];
                const float old_terr = terr[i];
                if (c > s1) {
                    float eroded = multipl * Kls * (c - s1);
                    s1 += eroded;
                    terr[i] -= eroded;
                    if (terr[i] < 0.0f) {
                        s1 += terr[i];
                        terr[i] = 0.0f;
                        cap += old_terr;
                    } else {
                        part.sed[i] = s1;
                        break;
                    }
                } else {
                    float deposit = multipl * Kld * (s1 - c);
                    s1 -= deposit;
                    terr[i] += deposit;
                }
                part.sed[i] = s1;
            }
            float conv = part.sed[0] * s.Kconv * s.d_t;
            part.sed[1] += conv;
            part.sed[0] -= conv;
            w.drops[id] = part;
            terr.z += 1e-5f * part.vol * multipl;
            terr.w = terr.x + terr.z + terr.y;
            mom.z += part.vol * part.vx * multipl;
            mom.w += part.vol * part.vy * multipl;
            H[w.id(cxs[k], cys[k])] = terr;
            M[w.id(cxs[k], cys[k])] = mom;
        }
    }
}

// glsl/smoothing.glsl:22-103 with the particle branch (:76-95): both layers,
// the drops' momentum folded into the momentum map, water display decay.
// Border texels copy their height and leave the momentum map's write buffer
// as it was.
void particle_smoothing_pass(World<float>& w, const OracleErosion& s) {
    const auto& H = w.height.rd();
    auto& Ho = w.height.wr();
    const auto& M = w.vel.rd();
    auto& Mo = w.vel.wr();
    const int n = w.n;
    const float count = (float)w.drops.size();
    for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x) {
            V4<float> terrain = H[w.id(x, y)];
            float tr = terrain.x, tg = terrain.y;
            if (x == 0 || y == 0 || x == n - 1 || y == n - 1) {
                Ho[w.id(x, y)] = terrain;
                continue;
            }
            V4<float> L4 = H[w.id(x - 1, y)], R4 = H[w.id(x + 1, y)], T4 = H[w.id(x, y + 1)], B4 = H[w.id(x, y - 1)];
            float lr = L4.x, lg = L4.y, rr = R4.x, rg = R4.y, trr = T4.x, tgg = T4.y, br = B4.x, bg = B4.y;
            float dlr = tr - lr, dlg = tg - lg; dlg += dlr;
            float drr = tr - rr, drg = tg - rg; drg += drr;
            float dtr = tr - trr, dtg = tg - tgg; dtg += dtr;
            float dbr = tr - br, dbg = tg - bg; dbg += dbr;
            float g_hdiff = std::fabs((dlg + drg + dtg + dbg) / 4.0f);
            float r_hdiff = std::fabs((dlr + drr + dtr + dbr) / 4.0f);
            float xr = dlr * drr, xg = dlg * drg, yr = dtr * dbr, yg = dtg * dbg;
            float nr = tr, ng = tg;
            if ((((-dlr) > r_hdiff || (-drr) > r_hdiff) && xr > 0) || (((-dtr) > r_hdiff || (-dbr) > r_hdiff) && yr > 0))
                nr = (tr + lr + rr + trr + br) / 5.0f;
            if ((((-dlg) > g_hdiff || (-drg) > g_hdiff) && xg > 0) || (((-dtg) > g_hdiff || (-dbg) > g_hdiff) && yg > 0))
                ng = (tg + lg + rg + tgg + bg) / 5.0f;
            float multip = gclamp(s.Kspeed[1] * s.d_t, 0.0f, 1.0f);
            V4<float> mom = M[w.id(x, y)];
            const float keep = gclamp(1.0f - 1e-12f * count, 0.0f, 1.0f);
            mom.x *= keep;
            mom.y *= keep;
            mom.x += 1e-12f * count * mom.z;
            mom.y += 1e-12f * count * mom.w;
            mom.z = 0.0f;
            mom.w = 0.0f;
            terrain.z *= gclamp(1.0f - 8e-8f * count, 0.0f, 1.0f);
            if (terrain.z < 1e-6f) terrain.z = 0.0f;
            if (std::sqrt(mom.x * mom.x + mom.y * mom.y) < 1e-12f) { mom.x = 0.0f; mom.y = 0.0f; }
            Mo[w.id(x, y)] = mom;
            terrain.x = multip * nr + (1.0f - multip) * terrain.x;
            terrain.y = multip * ng + (1.0f - multip) * terrain.y;
            terrain.w = terrain.x + terrain.y + terrain.z;
            Ho[w.id(x, y)] = terrain;
        }
    w.height.swap();
    w.vel.swap();
}

// Erosion::dispatch_particle (src/erosion.cpp:132-156): movement, erosion,
// thermal layers, smoothing
void particle_step(World<float>& w, const OracleErosion& s, const OracleOptions& o) {
    uint64_t n1 = w.step + 1;
    particle_move_pass(w, s, o.rain_mode != 0, n1, o.rain_seed);
    particle_erosion_pass(w, s);
    for (int layer = 0; layer < 2; ++layer) {
        if (o.skip_identity && s.Kspeed[layer] == 0.0f) continue;
        thermal_flux_pass(w, s, layer);
        thermal_transport_pass(w, layer);
    }
    particle_smoothing_pass(w, s);
    w.step = n1;
}

// ---- simplex fBm (own 2-D simplex, Gustavson 2005 "Simplex noise demystified")
inline uint32_t fmix32(uint32_t h) {  // MurmurHash3 finaliser (Appleby, public domain)
    h ^= h >> 16; h *= 0x85ebca6bu; h ^= h >> 13; h *= 0xc2b2ae35u; h ^= h >> 16;
    return h;
}
inline uint32_t corner_hash(int32_t i, int32_t j, uint32_t seed) {
    return fmix32((uint32_t)i * 0x8da6b343u ^ (uint32_t)j * 0xd8163841u ^ seed * 0xcb1ab31fu);
}
inline float grad_dot(uint32_t h, float x, float y) {
    // 8 gradient directions: (+-1,+-1), (+-1,0), (0,+-1)
    switch (h & 7u) {
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
inline float simplex2f(float x, float y, uint32_t seed) {
    const float F2 = 0.366025403784f;  // (sqrt(3)-1)/2
    const float G2 = 0.211324865405f;  // (3-sqrt(3))/6
    float s = (x + y) * F2;
    float fi = std::floor(x + s), fj = std::floor(y + s);
    float t = (fi + fj) * G2;
    float x0 = x - (fi - t), y0 = y - (fj - t);
    int i1 = x0 > y0 ? 1 : 0, j1 = 1 - i1;
    float x1 = x0 - (float)i1 + G2, y1 = y0 - (float)j1 + G2;
    float x2 = x0 - 1.0f + 2.0f * G2, y2 = y0 - 1.0f + 2.0f * G2;
    int32_t i = (int32_t)fi, j = (int32_t)fj;
    float n = 0.0f;
    float t0 = 0.5f - x0 * x0 - y0 * y0;
    if (t0 > 0.0f) { t0 = t0 * t0; n = n + t0 * t0 * grad_dot(corner_hash(i, j, seed), x0, y0); }
    float t1 = 0.5f - x1 * x1 - y1 * y1;
    if (t1 > 0.0f) { t1 = t1 * t1; n = n + t1 * t1 * grad_dot(corner_hash(i + i1, j + j1, seed), x1, y1); }
    float t2 = 0.5f - x2 * x2 - y2 * y2;
    if (t2 > 0.0f) { t2 = t2 * t2; n = n + t2 * t2 * grad_dot(corner_hash(i + 1, j + 1, seed), x2, y2); }
    return 70.0f * n;
}

}  // namespace

// ---- C interface (ctypes) ---------------------------------------------------
extern "C" {

enum { F_ROCK = 0, F_WATER, F_SED, F_FL, F_FR, F_FT, F_FB, F_U, F_V, F_DIRT, F_SED_DIRT, F_VZ, F_TOTAL, F_VW, F_COUNT };

struct OracleHandle {
    int prec;
    World<float>* wf;
    World<double>* wd;
};

void* hgo_create(int n, int precision) {
    if (n <= 0) return nullptr;
    auto* h = new OracleHandle{precision, nullptr, nullptr};
    if (precision == 64) h->wd = new World<double>(n);
    else h->wf = new World<float>(n);
    return h;
}

void hgo_destroy(void* p) {
    auto* h = (OracleHandle*)p;
    if (!h) return;
    delete h->wf;
    delete h->wd;
    delete h;
}

}  // extern "C"
template <typename T> static T* chan(World<T>& w, int field, size_t i, bool write) {
    (void)write;
    switch (field) {
        case F_ROCK: return &w.height.tex[w.height.r][i].x;
        case F_DIRT: return &w.height.tex[w.height.r][i].y;
        case F_WATER: return &w.height.tex[w.height.r][i].z;
        case F_TOTAL: return &w.height.tex[w.height.r][i].w;
        case F_SED: return &w.sed.tex[w.sed.r][i].x;
        case F_SED_DIRT: return &w.sed.tex[w.sed.r][i].y;
        case F_FL: return &w.flux.tex[w.flux.r][i].x;
        case F_FR: return &w.flux.tex[w.flux.r][i].y;
        case F_FT: return &w.flux.tex[w.flux.r][i].z;
        case F_FB: return &w.flux.tex[w.flux.r][i].w;
        case F_U: return &w.vel.tex[w.vel.r][i].x;
        case F_V: return &w.vel.tex[w.vel.r][i].y;
        case F_VZ: return &w.vel.tex[w.vel.r][i].z;
        case F_VW: return &w.vel.tex[w.vel.r][i].w;
    }
    return nullptr;
}

template <typename T> static int set_field(World<T>& w, int field, const double* src) {
    if (field < 0 || field >= F_COUNT) return -1;
    size_t c = (size_t)w.n * w.n;
    for (size_t i = 0; i < c; ++i) *chan(w, field, i, true) = (T)src[i];
    // keep the total channel consistent with rock + dirt + water, as every pass writes it
    if (field == F_ROCK || field == F_DIRT || field == F_WATER)
        for (size_t i = 0; i < c; ++i) {
            auto& t = w.height.tex[w.height.r][i];
            t.w = t.x + t.y + t.z;
        }
    return 0;
}

extern "C" {
int hgo_set_field(void* p, int field, const double* src) {
    auto* h = (OracleHandle*)p;
    return h->wd ? set_field(*h->wd, field, src) : set_field(*h->wf, field, src);
}

}  // extern "C"
template <typename T> static int get_field(World<T>& w, int field, double* dst) {
    if (field < 0 || field >= F_COUNT) return -1;
    size_t c = (size_t)w.n * w.n;
    for (size_t i = 0; i < c; ++i) dst[i] = (double)*chan(w, field, i, false);
    return 0;
}

extern "C" {
int hgo_get_field(void* p, int field, double* dst) {
    auto* h = (OracleHandle*)p;
    return h->wd ? get_field(*h->wd, field, dst) : get_field(*h->wf, field, dst);
}

int hgo_set_ks_field(void* p, const float* ks) {
    auto* h = (OracleHandle*)p;
    int n = h->wd ? h->wd->n : h->wf->n;
    std::vector<float>& dst = h->wd ? h->wd->ks : h->wf->ks;
    if (!ks) { dst.clear(); return 0; }
    dst.assign(ks, ks + (size_t)n * n);
    return 0;
}

void hgo_set_step(void* p, uint64_t step) {
    auto* h = (OracleHandle*)p;
    if (h->wd) h->wd->step = step; else h->wf->step = step;
}

uint64_t hgo_get_step(void* p) {
    auto* h = (OracleHandle*)p;
    return h->wd ? h->wd->step : h->wf->step;
}

int hgo_step(void* p, const OracleErosion* s, const OracleOptions* o, int nsteps) {
    auto* h = (OracleHandle*)p;
    if (!h || !s || !o || nsteps < 0) return -1;
    if (s->particle_count != 0) return -2;  // particle branch of smoothing is out of scope
    for (int k = 0; k < nsteps; ++k) {
        if (h->wd) one_step(*h->wd, *s, *o);
        else one_step(*h->wf, *s, *o);
    }
    return 0;
}

// particle mode (precision 32): `count` droplets, all idle
int hgo_particles_init(void* p, int count) {
    auto* h = (OracleHandle*)p;
    if (!h || !h->wf || count < 0) return -1;
    h->wf->drops.assign((size_t)count, World<float>::Drop{});
    return 0;
}

int hgo_particle_step(void* p, const OracleErosion* s, const OracleOptions* o, int nsteps) {
    auto* h = (OracleHandle*)p;
    if (!h || !h->wf || !s || !o || nsteps < 0) return -1;
    for (int k = 0; k < nsteps; ++k) particle_step(*h->wf, *s, *o);
    return 0;
}

// droplet state: 8 floats each (x, y, vx, vy, volume, rock sediment, dirt
// sediment, capacity) and iters / kill flag
int hgo_particles_get(void* p, float* state8, uint32_t* iters, int32_t* kill) {
    auto* h = (OracleHandle*)p;
    if (!h || !h->wf) return -1;
    for (size_t i = 0; i < h->wf->drops.size(); ++i) {
        const auto& d = h->wf->drops[i];
        float* o = state8 + 8 * i;
        o[0] = d.px; o[1] = d.py; o[2] = d.vx; o[3] = d.vy; o[4] = d.vol; o[5] = d.sed[0]; o[6] = d.sed[1]; o[7] = d.sc;
        iters[i] = d.iters;
        kill[i] = d.kill ? 1 : 0;
    }
    return 0;
}

// Single passes, for the per-pass unit tests.
// Restricts the grid passes to rows [lo, hi) (hi < 0: every row).
int hgo_set_rows(void* p, int lo, int hi) {
    auto* h = (OracleHandle*)p;
    const int n = h->wd ? h->wd->n : h->wf->n;
    if (lo < 0 || lo > n || (hi >= 0 && (hi < lo || hi > n))) return -1;
    if (h->wd) { h->wd->row_lo = lo; h->wd->row_hi = hi; }
    else { h->wf->row_lo = lo; h->wf->row_hi = hi; }
    return 0;
}

// Rows [y0, y1) of the current (read) texture `tex` (0 height, 1 flux,
// 2 velocity, 3 sediment, 4 thermal cross, 5 thermal diagonal), four
// channels per cell, to (write == 0) or from (write != 0) buf as doubles
// (float worlds convert exactly).  A slab decomposition's halo exchange.
int hgo_tex_rows(void* p, int tex, int y0, int y1, double* buf, int write) {
    auto* h = (OracleHandle*)p;
    auto run = [&](auto& w) -> int {
        using T = typename std::remove_reference<decltype(w.height.tex[0][0].x)>::type;
        if (y0 < 0 || y1 > w.n || y0 > y1) return -1;
        decltype(&w.height) pr = nullptr;
        switch (tex) {
            case 0: pr = &w.height; break;
            case 1: pr = &w.flux; break;
            case 2: pr = &w.vel; break;
            case 3: pr = &w.sed; break;
            case 4: pr = &w.thc; break;
            case 5: pr = &w.thd; break;
            default: return -1;
        }
        auto& t = pr->tex[pr->r];
        for (int y = y0; y < y1; ++y)
            for (int x = 0; x < w.n; ++x) {
                auto& v = t[w.id(x, y)];
                double* q = buf + 4 * ((size_t)(y - y0) * w.n + x);
                if (write) { v.x = (T)q[0]; v.y = (T)q[1]; v.z = (T)q[2]; v.w = (T)q[3]; }
                else { q[0] = v.x; q[1] = v.y; q[2] = v.z; q[3] = v.w; }
            }
        return 0;
    };
    return h->wd ? run(*h->wd) : run(*h->wf);
}

int hgo_pass(void* p, const OracleErosion* s, const OracleOptions* o, int which, int layer) {
    auto* h = (OracleHandle*)p;
    auto run = [&](auto& w) {
        switch (which) {
            case 0: rain_pass(w, *o, w.step + 1); break;
            case 1: flux_pass(w, *s); break;
            case 2: erosion_pass(w, *s); break;
            case 3: sediment_pass(w, *s); break;
            case 4: thermal_flux_pass(w, *s, layer); break;
            case 5: thermal_transport_pass(w, layer); break;
            case 6: smoothing_pass(w, *s); break;
            default: return -1;
        }
        return 0;
    };
    return h->wd ? run(*h->wd) : run(*h->wf);
}

// Thermal outflow textures of the last thermal_flux pass (8 channels per cell).
int hgo_get_thermal(void* p, double* cross4, double* diag4) {
    auto* h = (OracleHandle*)p;
    auto get = [&](auto& w) {
        size_t c = (size_t)w.n * w.n;
        for (size_t i = 0; i < c; ++i)
            for (int k = 0; k < 4; ++k) {
                cross4[4 * i + k] = (double)w.thc.rd()[i][k];
                diag4[4 * i + k] = (double)w.thd.rd()[i][k];
            }
        return 0;
    };
    return h->wd ? get(*h->wd) : get(*h->wf);
}

// FP64 totals: rock, dirt, water, sediment (rock + dirt channels)
void hgo_totals(void* p, double out[4]) {
    auto* h = (OracleHandle*)p;
    auto tot = [&](auto& w) {
        double r = 0, g = 0, b = 0, sd = 0;
        size_t c = (size_t)w.n * w.n;
        for (size_t i = 0; i < c; ++i) {
            const auto& t = w.height.rd()[i];
            const auto& s = w.sed.rd()[i];
            r += (double)t.x; g += (double)t.y; b += (double)t.z;
            sd += (double)s.x + (double)s.y;
        }
        out[0] = r; out[1] = g; out[2] = b; out[3] = sd;
    };
    if (h->wd) tot(*h->wd); else tot(*h->wf);
}

float hgo_atanf(float x) { return poly_atanf(x); }

// Sets the film guard depth (see g_film_guard); returns the previous one.
double hgo_set_film_guard(double depth) {
    double prev = g_film_guard;
    g_film_guard = depth;
    return prev;
}

// Selects the float instantiation's arctangent (see o_atan); returns the
// previous choice.
int hgo_set_float_atan_libm(int on) {
    int prev = g_float_atan_libm;
    g_float_atan_libm = on ? 1 : 0;
    return prev;
}

// Counts decreasing steps of poly_atanf over consecutive floats whose bit
// patterns lie in [lo_bits, hi_bits] (non-negative floats order like their bits).
uint64_t hgo_atan_monotone_violations(uint32_t lo_bits, uint32_t hi_bits) {
    uint64_t bad = 0;
    const int64_t chunk = 1 << 20;
    const int64_t total = (int64_t)hi_bits - (int64_t)lo_bits;
    #pragma omp parallel for schedule(dynamic) reduction(+ : bad)
    for (int64_t c0 = 0; c0 < total; c0 += chunk) {
        int64_t c1 = std::min(total, c0 + chunk);
        uint32_t b = lo_bits + (uint32_t)c0;
        float x;
        std::memcpy(&x, &b, 4);
        float prev = poly_atanf(x);
        for (int64_t k = c0 + 1; k <= c1; ++k) {
            b = lo_bits + (uint32_t)k;
            std::memcpy(&x, &b, 4);
            float cur = poly_atanf(x);
            if (cur < prev) ++bad;
            prev = cur;
        }
    }
    return bad;
}

void hgo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    philox4x32_10(ctr, key, out);
}

uint32_t hgo_rain_word(int x, int y, uint64_t step, uint32_t terrain, uint64_t seed) {
    return rain_word(x, y, step, terrain, seed);
}

float hgo_simplex2f(float x, float y, uint32_t seed) { return simplex2f(x, y, seed); }

// Raw fBm: sum over octaves of gain^o * simplex(x*f_o, y*f_o), f_o = freq*lac^o,
// octave o hashed with seed + o.  Cell (x, y) samples at integer coordinates.
void hgo_fbm_raw(float* out, int w, int hgt, uint32_t seed, int octaves, float freq, float lac, float gain) {
    OMP_ROWS
    for (int y = 0; y < hgt; ++y)
        for (int x = 0; x < w; ++x) {
            float sum = 0.0f, amp = 1.0f, f = freq;
            for (int o = 0; o < octaves; ++o) {
                sum = sum + amp * simplex2f((float)x * f, (float)y * f, seed + (uint32_t)o);
                amp = amp * gain;
                f = f * lac;
            }
            out[(size_t)y * w + x] = sum;
        }
}

// fBm min-max scaled into [lo, hi]: lo + ((v - min) / (max - min)) * (hi - lo)
void hgo_fbm_scaled(float* out, int n, uint32_t seed, int octaves, float freq, float lac, float gain,
                    float lo, float hi) {
    hgo_fbm_raw(out, n, n, seed, octaves, freq, lac, gain);
    size_t c = (size_t)n * n;
    float mn = out[0], mx = out[0];
    for (size_t i = 1; i < c; ++i) { mn = std::min(mn, out[i]); mx = std::max(mx, out[i]); }
    float range = mx - mn, span = hi - lo;
    for (size_t i = 0; i < c; ++i) out[i] = lo + ((out[i] - mn) / range) * span;
}

int hgo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void hgo_set_num_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

}  // extern "C"
