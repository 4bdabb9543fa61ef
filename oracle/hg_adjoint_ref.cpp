// FP64 reference adjoint of the single-material grid step — TEST
// INFRASTRUCTURE ONLY (checks the GPU adjoint; is itself checked against
// central finite differences of the oracle's FP64 forward).
//
// Forward model (one step, every field FP64, settings widened from float):
//   rain:      d_r = d + a                       (glsl/rain.glsl:48-53)
//   flux:      glsl/hydro_flux.glsl:77-166
//   erosion:   glsl/hydro_erosion.glsl:23-92 (rock layer; empty dirt layer)
//   sediment:  glsl/sediment_transport.glsl:66-93, img_interpolation.glsl:3-22
//   thermal:   glsl/thermal_erosion.glsl:28-109, glsl/thermal_transport.glsl:31-65
//              (layer 0, when Kspeed[0] != 0; the same double operations as
//              the oracle's thermal passes, with std::atan)
// Reverse mode with subgradients: max(0, x) and min(1, q) pass the
// derivative of the taken argument (ties take the constant side), clamps
// pass 0 when clamped, dissolve/deposit/exhaustion use the taken branch,
// floor() is locally constant, velocity and flux scale are locally constant
// in water films below kFilm; the talus marks are locally constant, the
// largest drop H and the steepest slope pass their derivative to the
// direction that attains them (the first in direction order).  Loss = mean((rock_final - target)^2);
// gradients with respect to the per-cell rock solubility Ks and the initial
// rock heights.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <utility>

namespace {

struct Params {
    double dt, G, EK, Kc, Kd0, Ke, amount, Kalpha, Kspeed;
    int period;
};

// Water films thinner than this (the float 5e-4 below which the erosion
// ignores the velocity, glsl/hydro_erosion.glsl:45-52) pass no adjoint
// through the velocity or the flux scale K (both derivatives grow like
// 1/depth).
const double kFilm = (double)5e-4f;

// thermal directions L, R, T, B, LT, RT, LB, RB
const int TOX[8] = {-1, 1, 0, 0, -1, 1, -1, 1};
const int TOY[8] = {0, 0, 1, -1, 1, 1, -1, -1};

struct State {
    std::vector<double> b, d, s, f[4];  // f: L, R, T, B
    void init(size_t c) {
        b.assign(c, 0); d.assign(c, 0); s.assign(c, 0);
        for (auto& x : f) x.assign(c, 0);
    }
};

// Intermediates of one forward step, kept for the reverse pass.
struct Inter {
    std::vector<double> dr, u, v, vz, d2, be, se;
};

const double FAR = 999999999999.0;

inline double gmax(double x, double y) { return x < y ? y : x; }
inline double gmin(double x, double y) { return y < x ? y : x; }

struct Model {
    int n;
    Params p;
    const float* ks;  // per-cell Ks (rock), float as the GPU holds it
    size_t id(int x, int y) const { return (size_t)y * n + x; }
    bool in(int x, int y) const { return x >= 0 && x < n && y >= 0 && y < n; }

    // Per-cell bodies of one step, shared by the full step and the windowed
    // finite-difference step (hgo_fd_ref).  The accessor `a` gives the step's
    // input at in-grid cells: a.b(x, y), a.d(x, y), a.s(x, y), a.f(k, x, y);
    // `rain` is the water added this step.
    template <class A>
    void flux_cell(const A& a, double rain, int x, int y, double fo[4], double& u, double& v, double& vz,
                   double& d2) const {
        auto w = [&](int xx, int yy) { return in(xx, yy) ? a.b(xx, yy) + (a.d(xx, yy) + rain) : FAR; };
        auto F = [&](int k, int xx, int yy) { return in(xx, yy) ? a.f(k, xx, yy) : 0.0; };
        double d1 = a.d(x, y) + rain;
        double wc = a.b(x, y) + d1;
        const int ox[4] = {-1, 1, 0, 0}, oy[4] = {0, 0, 1, -1};
        double g[4], fc[4];
        for (int k = 0; k < 4; ++k) {
            fc[k] = a.f(k, x, y);
            double ft = p.EK * fc[k] + p.dt * (p.G * (wc - w(x + ox[k], y + oy[k])));
            g[k] = gmax(0.0, ft);
        }
        if (x <= 0) g[0] = 0; else if (x >= n - 1) g[1] = 0;
        if (y <= 0) g[3] = 0; else if (y >= n - 1) g[2] = 0;
        double inl = F(1, x - 1, y), inr = F(0, x + 1, y), it = F(3, x, y + 1), ib = F(2, x, y - 1);
        double sum_in = inl + inr + it + ib;
        double sum_out = g[0] + g[1] + g[2] + g[3];
        double K = gmin(1.0, d1 / (sum_out * p.dt));
        for (int k = 0; k < 4; ++k) fo[k] = g[k] * K;
        d2 = gmax(0.0, d1 + p.dt * (sum_in - sum_out * K));
        vz = d1 + d2;
        u = 0; v = 0;
        if (vz > 0) {
            u = (inl - fc[0] + fc[1] - inr) / vz;
            v = (ib - fc[3] + fc[2] - it) / vz;
        }
    }

    template <class A>
    void erosion_cell(const A& a, int x, int y, double u, double v, double vz, float ks_cell, double& be,
                      double& se) const {
        auto B = [&](int xx, int yy) { return in(xx, yy) ? a.b(xx, yy) : 0.0; };
        double len = std::sqrt(u * u + v * v), ero = len;
        if (vz < 1e-3) {
            double dd = gmax(5e-4, vz);
            double t = gmin(gmax((dd - 1e-3) / (5e-4 - 1e-3), 0.0), 1.0);
            ero = len * (1 - t * t * (3 - 2 * t));
        }
        double dx = B(x + 1, y) - B(x - 1, y), dz = B(x, y + 1) - B(x, y - 1);
        double L3 = std::sqrt(4 * dx * dx + 16 + 4 * dz * dz);
        double ny = -4 / L3;
        double sa = gmax(0.02, std::sqrt(1 - ny * ny));
        double cc = gmax(0.0, p.Kc * sa * ero);
        double Kls = p.dt * (double)ks_cell, b = a.b(x, y), s = a.s(x, y);
        if (cc > s) {
            double del = Kls * (cc - s);
            b -= del; s += del;
            if (b < 0) { s += b; b = 0; }
        } else {
            double del = (p.dt * p.Kd0) * (s - cc);
            b += del; s -= del;
        }
        be = b; se = s;
    }

    // Lower-left tap of the sediment back-trace and its weights.
    void backtrace(int x, int y, double u, double v, int& ix, int& iy, double& fx, double& fy) const {
        double px = gmin(gmax(x - u * p.dt, 0.0), (double)(n - 1));
        double py = gmin(gmax(y - v * p.dt, 0.0), (double)(n - 1));
        ix = (int)px; iy = (int)py;
        fx = px - std::floor(px); fy = py - std::floor(py);
    }

    // Bilinear gather of eroded sediment se_at(x, y) (in-grid cells).
    template <class S>
    double sediment_cell(const S& se_at, int x, int y, double u, double v) const {
        int ix, iy;
        double fx, fy;
        backtrace(x, y, u, v, ix, iy, fx, fy);
        auto S_ = [&](int xx, int yy) { return in(xx, yy) ? se_at(xx, yy) : 0.0; };
        double v1 = S_(ix, iy) * (1 - fx) + S_(ix + 1, iy) * fx;
        double v2 = S_(ix, iy + 1) * (1 - fx) + S_(ix + 1, iy + 1) * fx;
        return v1 * (1 - fy) + v2 * fy;
    }

    double rain_of(uint64_t step1) const {
        return p.period > 0 && step1 % (uint64_t)p.period == 0 ? p.amount : 0.0;
    }

    struct FullIn {
        const State& X;
        size_t n;
        double b(int x, int y) const { return X.b[(size_t)y * n + x]; }
        double d(int x, int y) const { return X.d[(size_t)y * n + x]; }
        double s(int x, int y) const { return X.s[(size_t)y * n + x]; }
        double f(int k, int x, int y) const { return X.f[k][(size_t)y * n + x]; }
    };

    void step(const State& X, uint64_t step1, State& Y, Inter& I) const {
        const size_t c = (size_t)n * n;
        Y.init(c);
        I.dr.assign(c, 0); I.u.assign(c, 0); I.v.assign(c, 0); I.vz.assign(c, 0); I.d2.assign(c, 0);
        I.be.assign(c, 0); I.se.assign(c, 0);
        const double rain = rain_of(step1);
        const FullIn a{X, (size_t)n};
        for (size_t i = 0; i < c; ++i) I.dr[i] = X.d[i] + rain;
#pragma omp parallel for schedule(static)
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                size_t i = id(x, y);
                double fo[4];
                flux_cell(a, rain, x, y, fo, I.u[i], I.v[i], I.vz[i], I.d2[i]);
                for (int k = 0; k < 4; ++k) Y.f[k][i] = fo[k];
            }
        // erosion
#pragma omp parallel for schedule(static)
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                size_t i = id(x, y);
                erosion_cell(a, x, y, I.u[i], I.v[i], I.vz[i], ks[i], I.be[i], I.se[i]);
            }
        // sediment transport + evaporation
        auto se_at = [&](int xx, int yy) { return I.se[id(xx, yy)]; };
#pragma omp parallel for schedule(static)
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                size_t i = id(x, y);
                Y.s[i] = sediment_cell(se_at, x, y, I.u[i], I.v[i]);
                Y.d[i] = I.d2[i] * (1 - p.Ke * p.dt);
                Y.b[i] = I.be[i];
            }
        if (p.Kspeed != 0.0) thermal(I.be, Y.b);
    }

    // Talus outflows of cell (x, y) of rock field b (the oracle's
    // thermal_flux_pass for layer 0, in the same double operations).
    struct Talus {
        double dh[8], o[8], bk = 0, Hmax = 0, S = 0, s1 = 1, slope = 0;
        bool mk[8], sharp_taken = false;
        int jh = -1, js = -1;
    };
    Talus talus(const std::vector<double>& b, int x, int y) const {
        Talus t;
        const double FARH = 999999999999.0, bc = b[id(x, y)];
        for (int k = 0; k < 8; ++k) {
            int xx = x + TOX[k], yy = y + TOY[k];
            t.dh[k] = 0.0 + (bc - (in(xx, yy) ? b[id(xx, yy)] : FARH));
        }
        for (int k = 0; k < 8; ++k)
            if (t.dh[k] > t.Hmax) { t.Hmax = t.dh[k]; t.jh = k; }
        double Hh = gmin(bc, t.Hmax);
        double best_alph = -1e300;
        for (int k = 0; k < 8; ++k) {
            t.mk[k] = false;
            double bb = t.dh[k];
            if (bb <= 0) continue;
            double d = 1.0;
            if (k >= 4) d *= std::sqrt(2.0);
            double alph = std::atan(bb / d);
            if (alph > p.Kalpha) {
                double newsh = 1.0 + alph - p.Kalpha;
                if (newsh > t.s1) { t.s1 = newsh; t.sharp_taken = true; }
                if (alph > best_alph) { best_alph = alph; t.js = k; t.slope = bb / d; }
                t.bk += bb;
                t.mk[k] = true;
            }
        }
        double sh = t.s1;
        sh *= sh * sh;
        t.S = p.dt * p.Kspeed * sh * 1.0 * Hh / 2.0;
        for (int k = 0; k < 8; ++k) t.o[k] = t.mk[k] ? t.S * t.dh[k] / t.bk : 0.0;
        return t;
    }

    // thermal_erosion + thermal_transport, layer 0
    void thermal(const std::vector<double>& b, std::vector<double>& out) const {
        const size_t c = (size_t)n * n;
        std::vector<double> o(8 * c);
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                Talus t = talus(b, x, y);
                for (int k = 0; k < 8; ++k) o[8 * id(x, y) + k] = t.o[k];
            }
        const int opp[8] = {1, 0, 3, 2, 7, 6, 5, 4};
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                size_t i = id(x, y);
                double in_flux = 0;
                for (int k = 0; k < 8; ++k) {
                    int xx = x + TOX[k], yy = y + TOY[k];
                    in_flux += in(xx, yy) ? o[8 * id(xx, yy) + opp[k]] : 0.0;
                }
                double sum = 0;
                for (int k = 0; k < 8; ++k) sum -= o[8 * i + k];
                sum += in_flux;
                out[i] = b[i] + sum;
            }
    }

    // Reverse of the thermal passes: A_out is d(loss)/d(rock after thermal),
    // G receives d(loss)/d(rock before thermal).
    void thermal_reverse(const std::vector<double>& b, const std::vector<double>& A_out,
                         std::vector<double>& G) const {
        const size_t c = (size_t)n * n;
        G = A_out;
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                Talus t = talus(b, x, y);
                if (t.bk == 0.0) continue;  // no marked direction
                size_t i = id(x, y);
                double gk[8], gavg = 0;
                for (int k = 0; k < 8; ++k) {
                    gk[k] = 0;
                    if (!t.mk[k]) continue;
                    gk[k] = A_out[id(x + TOX[k], y + TOY[k])] - A_out[i];
                    gavg += gk[k] * t.dh[k];
                }
                gavg /= t.bk;
                double gdh[8] = {0, 0, 0, 0, 0, 0, 0, 0}, gb = 0;
                for (int k = 0; k < 8; ++k)
                    if (t.mk[k]) gdh[k] = t.S / t.bk * (gk[k] - gavg);
                const double dS = gavg;
                const double sh3 = t.s1 * t.s1 * t.s1;
                const double Hh = gmin(b[i], t.Hmax);
                const double dH = dS * p.dt * p.Kspeed * sh3 / 2.0;
                if (t.sharp_taken && t.js >= 0) {
                    double ds1 = dS * p.dt * p.Kspeed * Hh / 2.0 * 3.0 * t.s1 * t.s1;
                    double dslope = ds1 / (1.0 + t.slope * t.slope);
                    gdh[t.js] += dslope / (t.js >= 4 ? std::sqrt(2.0) : 1.0);
                }
                if (t.Hmax < b[i]) { if (t.jh >= 0) gdh[t.jh] += dH; }
                else gb += dH;
                double own = gb;
                for (int k = 0; k < 8; ++k) {
                    own += gdh[k];
                    int xx = x + TOX[k], yy = y + TOY[k];
                    if (in(xx, yy)) G[id(xx, yy)] -= gdh[k];
                }
                G[i] += own;
            }
        (void)c;
    }

    // Reverse of one step: A holds d(loss)/d(outputs of the step) and is
    // replaced by d(loss)/d(inputs); dKs accumulates.
    void reverse(const State& X, uint64_t step1, State& A, std::vector<double>& dKs) const {
        const size_t c = (size_t)n * n;
        State Y;
        Inter I;
        step(X, step1, Y, I);
        State R;  // input adjoints
        R.init(c);
        std::vector<double> dse(c, 0), du(c, 0), dv(c, 0), dvz(c, 0), dd2(c, 0), ddr(c, 0);
        const double evap = 1 - p.Ke * p.dt;
        // thermal: the adjoint of the eroded rock
        std::vector<double> Abe = A.b;
        if (p.Kspeed != 0.0) thermal_reverse(I.be, A.b, Abe);
        // sediment transport
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                size_t i = id(x, y);
                dd2[i] += A.d[i] * evap;
                double a = A.s[i];
                double rx = x - I.u[i] * p.dt, ry = y - I.v[i] * p.dt;
                double px = gmin(gmax(rx, 0.0), (double)(n - 1));
                double py = gmin(gmax(ry, 0.0), (double)(n - 1));
                int ix = (int)px, iy = (int)py;
                double fx = px - std::floor(px), fy = py - std::floor(py);
                auto S = [&](int xx, int yy) { return in(xx, yy) ? I.se[id(xx, yy)] : 0.0; };
                auto add = [&](int xx, int yy, double val) { if (in(xx, yy)) dse[id(xx, yy)] += val; };
                add(ix, iy, a * (1 - fx) * (1 - fy));
                add(ix + 1, iy, a * fx * (1 - fy));
                add(ix, iy + 1, a * (1 - fx) * fy);
                add(ix + 1, iy + 1, a * fx * fy);
                double dfx = (S(ix + 1, iy) - S(ix, iy)) * (1 - fy) + (S(ix + 1, iy + 1) - S(ix, iy + 1)) * fy;
                double dfy = (S(ix, iy + 1) * (1 - fx) + S(ix + 1, iy + 1) * fx) - (S(ix, iy) * (1 - fx) + S(ix + 1, iy) * fx);
                bool cx = rx > 0.0 && rx < (double)(n - 1), cy = ry > 0.0 && ry < (double)(n - 1);
                if (cx) du[i] += a * dfx * (-p.dt);
                if (cy) dv[i] += a * dfy * (-p.dt);
            }
        // erosion
        std::vector<double> pdx(c, 0), pdz(c, 0);
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                size_t i = id(x, y);
                auto B = [&](int xx, int yy) { return in(xx, yy) ? X.b[id(xx, yy)] : 0.0; };
                double u = I.u[i], v = I.v[i], vz = I.vz[i];
                double len = std::sqrt(u * u + v * v), ero = len, dero_dlen = 1, dero_dvz = 0;
                if (vz < 1e-3) {
                    double dd = gmax(5e-4, vz);
                    double tr = (dd - 1e-3) / (5e-4 - 1e-3);
                    double t = gmin(gmax(tr, 0.0), 1.0);
                    double sm = t * t * (3 - 2 * t);
                    ero = len * (1 - sm);
                    dero_dlen = 1 - sm;
                    if (vz > 5e-4 && tr > 0 && tr < 1) dero_dvz = -len * 6 * t * (1 - t) / (5e-4 - 1e-3);
                }
                double dx = B(x + 1, y) - B(x - 1, y), dz = B(x, y + 1) - B(x, y - 1);
                double L3 = std::sqrt(4 * dx * dx + 16 + 4 * dz * dz);
                double ny = -4 / L3;
                double sin_a = std::sqrt(1 - ny * ny);
                double sa = gmax(0.02, sin_a);
                double craw = p.Kc * sa * ero;
                double cc = gmax(0.0, craw);
                double Kls = p.dt * (double)ks[i], Kld = p.dt * p.Kd0, b = X.b[i], s = X.s[i];
                double ab = Abe[i], as = dse[i];
                double gb = 0, gs = 0, gc = 0, gK = 0;
                if (cc > s) {
                    double del = Kls * (cc - s);
                    if (b - del < 0) {  // exhausted: b' = 0, s' = s + b
                        gb = as; gs = as;
                    } else {
                        gb = ab; gs = ab * Kls + as * (1 - Kls);
                        gc = -ab * Kls + as * Kls;
                        gK = (-ab + as) * (cc - s);
                    }
                } else {
                    gb = ab; gs = ab * Kld + as * (1 - Kld);
                    gc = -ab * Kld + as * Kld;
                }
                dKs[i] += gK * p.dt;
                R.b[i] += gb;
                R.s[i] += gs;
                if (craw > 0) {
                    double gsa = gc * p.Kc * ero, gero = gc * p.Kc * sa;
                    if (sin_a > 0.02) {
                        double gny = gsa * (-ny / sin_a);
                        double gL3 = gny * (4 / (L3 * L3));
                        pdx[i] = gL3 * 4 * dx / L3;
                        pdz[i] = gL3 * 4 * dz / L3;
                    }
                    double glen = gero * dero_dlen;
                    dvz[i] += gero * dero_dvz;
                    if (len > 0) { du[i] += glen * u / len; dv[i] += glen * v / len; }
                }
            }
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                size_t i = id(x, y);
                if (in(x + 1, y)) R.b[id(x + 1, y)] += pdx[i];
                if (in(x - 1, y)) R.b[id(x - 1, y)] -= pdx[i];
                if (in(x, y + 1)) R.b[id(x, y + 1)] += pdz[i];
                if (in(x, y - 1)) R.b[id(x, y - 1)] -= pdz[i];
            }
        // flux
        auto w = [&](int x, int y) { return in(x, y) ? X.b[id(x, y)] + I.dr[id(x, y)] : FAR; };
        auto F = [&](int k, int x, int y) { return in(x, y) ? X.f[k][id(x, y)] : 0.0; };
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                size_t i = id(x, y);
                const int ox[4] = {-1, 1, 0, 0}, oy[4] = {0, 0, 1, -1};
                double wc = w(x, y), d1 = I.dr[i];
                double ft[4], g[4];
                bool zero[4] = {false, false, false, false};
                for (int k = 0; k < 4; ++k) {
                    ft[k] = p.EK * X.f[k][i] + p.dt * (p.G * (wc - w(x + ox[k], y + oy[k])));
                    g[k] = gmax(0.0, ft[k]);
                }
                if (x <= 0) zero[0] = true; else if (x >= n - 1) zero[1] = true;
                if (y <= 0) zero[3] = true; else if (y >= n - 1) zero[2] = true;
                for (int k = 0; k < 4; ++k) if (zero[k]) g[k] = 0;
                double inl = F(1, x - 1, y), inr = F(0, x + 1, y), it = F(3, x, y + 1), ib = F(2, x, y - 1);
                double sum_in = inl + inr + it + ib;
                double sum_out = g[0] + g[1] + g[2] + g[3];
                double den = sum_out * p.dt;
                double q = d1 / den;
                double K = gmin(1.0, q);
                double arg = d1 + p.dt * (sum_in - sum_out * K);
                double d2 = gmax(0.0, arg);
                double vz = d1 + d2;
                double u = I.u[i], v = I.v[i];
                // velocity
                double gvz = dvz[i], gin[4] = {0, 0, 0, 0}, gfown[4] = {0, 0, 0, 0};
                if (vz >= kFilm) {  // thinner films: velocity locally constant
                    gin[0] += du[i] / vz; gin[1] -= du[i] / vz;
                    gfown[0] -= du[i] / vz; gfown[1] += du[i] / vz;
                    gin[3] += dv[i] / vz; gin[2] -= dv[i] / vz;
                    gfown[3] -= dv[i] / vz; gfown[2] += dv[i] / vz;
                    gvz -= (du[i] * u + dv[i] * v) / vz;
                }
                double gd1 = gvz, gd2 = gvz + dd2[i];
                double garg = arg > 0 ? gd2 : 0;
                gd1 += garg;
                double gsum_in = p.dt * garg, gsum_outK = -p.dt * garg;
                for (int k = 0; k < 4; ++k) gin[k] += gsum_in;
                double gK = gsum_outK * sum_out, gsum_out = gsum_outK * K;
                for (int k = 0; k < 4; ++k) gK += A.f[k][i] * g[k];
                double gg[4];
                for (int k = 0; k < 4; ++k) gg[k] = A.f[k][i] * K + gsum_out;
                if (q < 1.0 && d1 >= kFilm) {  // K = q; thinner films: K locally constant
                    gd1 += gK / den;
                    double gden = -gK * d1 / (den * den);
                    for (int k = 0; k < 4; ++k) gg[k] += gden * p.dt;
                }
                double gw = 0;
                for (int k = 0; k < 4; ++k) {
                    if (zero[k] || !(ft[k] > 0)) continue;
                    gfown[k] += p.EK * gg[k];
                    double gdh = p.dt * p.G * gg[k];
                    gw += gdh;
                    int xx = x + ox[k], yy = y + oy[k];
                    if (in(xx, yy)) { R.b[id(xx, yy)] -= gdh; ddr[id(xx, yy)] -= gdh; }
                }
                R.b[i] += gw;
                ddr[i] += gw + gd1;
                for (int k = 0; k < 4; ++k) R.f[k][i] += gfown[k];
                // inflows are the neighbours' old facing fluxes
                if (in(x - 1, y)) R.f[1][id(x - 1, y)] += gin[0];
                if (in(x + 1, y)) R.f[0][id(x + 1, y)] += gin[1];
                if (in(x, y + 1)) R.f[3][id(x, y + 1)] += gin[2];
                if (in(x, y - 1)) R.f[2][id(x, y - 1)] += gin[3];
            }
        for (size_t i = 0; i < c; ++i) R.d[i] = ddr[i];  // rain adds a constant
        A = R;
    }
};

}  // namespace

extern "C" {

// settings: dt, G, ENERGY_KEPT, Kc, Kd[0], Ke, rain amount, Kalpha[0],
// Kspeed[0] (floats as the UBO holds them), rain period.  Inputs n*n
// doubles/floats; outputs n*n doubles.
int hgo_adjoint_ref(int n, const float* settings, int period, uint64_t step0, int nsteps, const double* b0,
                    const float* ks, const double* target, double* loss, double* dKs, double* db0) {
    if (n <= 0 || nsteps < 0) return -1;
    Model m;
    m.n = n;
    m.p = Params{settings[0], settings[1], settings[2], settings[3], settings[4],
                 settings[5], settings[6], settings[7], settings[8], period};
    m.ks = ks;
    const size_t c = (size_t)n * n;
    std::vector<State> tape(nsteps + 1);
    tape[0].init(c);
    for (size_t i = 0; i < c; ++i) tape[0].b[i] = b0[i];
    for (int k = 0; k < nsteps; ++k) {
        Inter I;
        m.step(tape[k], step0 + k + 1, tape[k + 1], I);
    }
    double L = 0;
    State A;
    A.init(c);
    for (size_t i = 0; i < c; ++i) {
        double e = tape[nsteps].b[i] - target[i];
        L += e * e;
        A.b[i] = 2 * e / (double)c;
    }
    *loss = L / (double)c;
    std::vector<double> g(c, 0);
    for (int k = nsteps - 1; k >= 0; --k) m.reverse(tape[k], step0 + k + 1, A, g);
    for (size_t i = 0; i < c; ++i) { dKs[i] = g[i]; db0[i] = A.b[i]; }
    return 0;
}

// Forward only (same model), for finite differences on the reference itself.
int hgo_forward_ref(int n, const float* settings, int period, uint64_t step0, int nsteps, const double* b0,
                    const float* ks, double* b_out) {
    Model m;
    m.n = n;
    m.p = Params{settings[0], settings[1], settings[2], settings[3], settings[4],
                 settings[5], settings[6], settings[7], settings[8], period};
    m.ks = ks;
    const size_t c = (size_t)n * n;
    State X, Y;
    X.init(c);
    for (size_t i = 0; i < c; ++i) X.b[i] = b0[i];
    Inter I;  // buffers reused across steps (step() overwrites every element)
    for (int k = 0; k < nsteps; ++k) {
        m.step(X, step0 + k + 1, Y, I);
        std::swap(X, Y);
    }
    for (size_t i = 0; i < c; ++i) b_out[i] = X.b[i];
    return 0;
}

// Central finite differences of loss = mean((rock_final - target)^2) after
// nsteps of the same FP64 model, one per (cell, parameter) pair: parameter
// 0 perturbs the cell's Ks by +-eps (rounded to float, as the field is
// held; h is the rounded difference), parameter 1 its initial rock by
// +-eps.  out[j] = (L(+) - L(-)) / h, the loss difference summed as
// (bp - bm)(bp + bm - 2 t) per cell, which does not cancel the way
// L(+) - L(-) does.
//
// Exact and windowed: every perturbed forward runs in lockstep with one
// unperturbed (baseline) forward and holds its own state only on a
// rectangle R outside of which it equals the baseline.  One step moves a
// difference by at most one cell through the flux, water, velocity and
// erosion (their stencils are the 4-neighbourhood), so the step's
// intermediates can differ only on R1 = R grown by one cell; the sediment
// gather then reads eroded sediment that differs only on R1, which reaches
// a cell outside R1 only through that cell's back-trace taps.  The new R is
// R grown by two cells plus every cell whose (baseline) taps touch R1:
// those with taps within their own 3 x 3 neighbourhood lie in R grown by
// two, the others come from a per-step list of far-reaching back-traces.
// The per-cell arithmetic is the full step's own (flux_cell, erosion_cell,
// sediment_cell), so each perturbed forward equals the full forward of the
// perturbed inputs bit for bit (tests/test_adjoint_reference.py checks it).
// Talus slippage (Kspeed[0] != 0) moves rock two cells per step through
// the 8-neighbourhood; it is not windowed: those runs fall back to full
// forwards.
}  // extern "C"

// Helpers of hgo_fd_ref (C++ linkage, file-local).
namespace {

struct Rect {
    int x0, y0, x1, y1;  // inclusive
    bool has(int x, int y) const { return x >= x0 && x <= x1 && y >= y0 && y <= y1; }
    int w() const { return x1 - x0 + 1; }
    int h() const { return y1 - y0 + 1; }
    size_t at(int x, int y) const { return (size_t)(y - y0) * w() + (x - x0); }
    Rect grow(int r, int n) const {
        return Rect{std::max(0, x0 - r), std::max(0, y0 - r), std::min(n - 1, x1 + r), std::min(n - 1, y1 + r)};
    }
    void add(int x, int y) {
        x0 = std::min(x0, x); y0 = std::min(y0, y); x1 = std::max(x1, x); y1 = std::max(y1, y);
    }
};

// One perturbed forward: its state on R (fields b, d, s, f) and its Ks cell.
struct Perturbed {
    Rect R;
    std::vector<double> b, d, s, f[4];
    int kx = -1, ky = -1;  // the cell whose Ks is perturbed (-1: none)
    float kval = 0;
};

// A back-trace whose lower-left tap (ix, iy) leaves the cell's 3 x 3
// neighbourhood.
struct Far {
    int x, y, ix, iy;
};

Perturbed start(const double* b0, const float* ks, int n, int cell, int param, double delta) {
    Perturbed q;
    const int x = cell % n, y = cell / n;
    q.R = Rect{x, y, x, y};
    q.b = {b0[cell]};
    q.d = {0.0};
    q.s = {0.0};
    for (auto& f : q.f) f = {0.0};
    if (param == 0) {
        q.kx = x; q.ky = y;
        q.kval = (float)((double)ks[cell] + delta);
    } else {
        q.b[0] = b0[cell] + delta;
    }
    return q;
}

// Baseline step X -> Y (intermediates in I) and its far-reaching back-traces.
void baseline_step(const Model& mdl, const State& X, uint64_t step1, State& Y, Inter& I, std::vector<Far>& far) {
    const int n = mdl.n;
    mdl.step(X, step1, Y, I);
    far.clear();
    for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x) {
            const size_t i = (size_t)y * n + x;
            int ix, iy;
            double fx, fy;
            mdl.backtrace(x, y, I.u[i], I.v[i], ix, iy, fx, fy);
            if (ix < x - 1 || ix > x || iy < y - 1 || iy > y) far.push_back(Far{x, y, ix, iy});
        }
}

// Advances q by the step the baseline took from X to Y (intermediates I).
void advance(const Model& mdl, Perturbed& q, const State& X, const State& Y, const Inter& I,
             const std::vector<Far>& far, double rain) {
    const int n = mdl.n;
    struct In {  // the step's input: q's own state on R, the baseline's elsewhere
        const Perturbed& q;
        const State& X;
        int n;
        double b(int x, int y) const { return q.R.has(x, y) ? q.b[q.R.at(x, y)] : X.b[(size_t)y * n + x]; }
        double d(int x, int y) const { return q.R.has(x, y) ? q.d[q.R.at(x, y)] : X.d[(size_t)y * n + x]; }
        double s(int x, int y) const { return q.R.has(x, y) ? q.s[q.R.at(x, y)] : X.s[(size_t)y * n + x]; }
        double f(int k, int x, int y) const {
            return q.R.has(x, y) ? q.f[k][q.R.at(x, y)] : X.f[k][(size_t)y * n + x];
        }
    } in{q, X, n};
    const Rect R = q.R, R1 = R.grow(1, n);
    const size_t c1 = (size_t)R1.w() * R1.h();
    std::vector<double> pf[4], pu(c1), pv(c1), pd2(c1), pbe(c1), pse(c1);
    for (auto& f : pf) f.resize(c1);
    for (int y = R1.y0; y <= R1.y1; ++y)
        for (int x = R1.x0; x <= R1.x1; ++x) {
            const size_t l = R1.at(x, y);
            double fo[4], vz;
            mdl.flux_cell(in, rain, x, y, fo, pu[l], pv[l], vz, pd2[l]);
            for (int k = 0; k < 4; ++k) pf[k][l] = fo[k];
            const float kc = (x == q.kx && y == q.ky) ? q.kval : mdl.ks[(size_t)y * n + x];
            mdl.erosion_cell(in, x, y, pu[l], pv[l], vz, kc, pbe[l], pse[l]);
        }
    // E: the cells of R1 whose eroded sediment differs from the baseline's;
    // only back-traces with a tap in E can change a sediment outside R1
    Rect E{n, n, -1, -1};
    for (int y = R1.y0; y <= R1.y1; ++y)
        for (int x = R1.x0; x <= R1.x1; ++x)
            if (pse[R1.at(x, y)] != I.se[(size_t)y * n + x]) E.add(x, y);
    Rect R2 = R.grow(2, n);
    if (E.x1 >= 0)
        for (const Far& fr : far)
            if (!R1.has(fr.x, fr.y) && fr.ix <= E.x1 && fr.ix + 1 >= E.x0 && fr.iy <= E.y1 && fr.iy + 1 >= E.y0)
                R2.add(fr.x, fr.y);
    const size_t c2 = (size_t)R2.w() * R2.h();
    Perturbed nq;
    nq.R = R2;
    nq.kx = q.kx; nq.ky = q.ky; nq.kval = q.kval;
    nq.b.resize(c2); nq.d.resize(c2); nq.s.resize(c2);
    for (auto& f : nq.f) f.resize(c2);
    auto se_at = [&](int xx, int yy) { return R1.has(xx, yy) ? pse[R1.at(xx, yy)] : I.se[(size_t)yy * n + xx]; };
    const double evap = 1 - mdl.p.Ke * mdl.p.dt;
    for (int y = R2.y0; y <= R2.y1; ++y)
        for (int x = R2.x0; x <= R2.x1; ++x) {
            const size_t l2 = R2.at(x, y), i = (size_t)y * n + x;
            if (R1.has(x, y)) {
                const size_t l = R1.at(x, y);
                nq.s[l2] = mdl.sediment_cell(se_at, x, y, pu[l], pv[l]);
                nq.d[l2] = pd2[l] * evap;
                nq.b[l2] = pbe[l];
                for (int k = 0; k < 4; ++k) nq.f[k][l2] = pf[k][l];
            } else {
                nq.s[l2] = mdl.sediment_cell(se_at, x, y, I.u[i], I.v[i]);
                nq.d[l2] = Y.d[i];
                nq.b[l2] = Y.b[i];
                for (int k = 0; k < 4; ++k) nq.f[k][l2] = Y.f[k][i];
            }
        }
    // keep the state only where it differs from the baseline's (the rest is
    // the baseline's by value); the Ks cell stays inside
    Rect D{n, n, -1, -1};
    if (q.kx >= 0) D.add(q.kx, q.ky);
    for (int y = R2.y0; y <= R2.y1; ++y)
        for (int x = R2.x0; x <= R2.x1; ++x) {
            const size_t l2 = R2.at(x, y), i = (size_t)y * n + x;
            bool same = nq.b[l2] == Y.b[i] && nq.d[l2] == Y.d[i] && nq.s[l2] == Y.s[i];
            for (int k = 0; k < 4; ++k) same = same && nq.f[k][l2] == Y.f[k][i];
            if (!same) D.add(x, y);
        }
    if (D.x1 < 0) D = Rect{R2.x0, R2.y0, R2.x0, R2.y0};  // no difference left: keep one cell
    if (D.x0 == R2.x0 && D.y0 == R2.y0 && D.x1 == R2.x1 && D.y1 == R2.y1) {
        q = std::move(nq);
        return;
    }
    Perturbed sq;
    sq.R = D;
    sq.kx = q.kx; sq.ky = q.ky; sq.kval = q.kval;
    const size_t cd = (size_t)D.w() * D.h();
    sq.b.resize(cd); sq.d.resize(cd); sq.s.resize(cd);
    for (auto& f : sq.f) f.resize(cd);
    for (int y = D.y0; y <= D.y1; ++y)
        for (int x = D.x0; x <= D.x1; ++x) {
            const size_t l = D.at(x, y), l2 = R2.at(x, y);
            sq.b[l] = nq.b[l2]; sq.d[l] = nq.d[l2]; sq.s[l] = nq.s[l2];
            for (int k = 0; k < 4; ++k) sq.f[k][l] = nq.f[k][l2];
        }
    q = std::move(sq);
}

Model make_model(int n, const float* settings, int period, const float* ks) {
    Model mdl;
    mdl.n = n;
    mdl.p = Params{settings[0], settings[1], settings[2], settings[3], settings[4],
                   settings[5], settings[6], settings[7], settings[8], period};
    mdl.ks = ks;
    return mdl;
}

// Runs the perturbed forwards qs in lockstep with the baseline from b0;
// X ends as the baseline's final state.
void run_windowed(const Model& mdl, const double* b0, uint64_t step0, int nsteps, std::vector<Perturbed>& qs,
                  State& X) {
    const size_t c = (size_t)mdl.n * mdl.n;
    State Y;
    X.init(c);
    for (size_t i = 0; i < c; ++i) X.b[i] = b0[i];
    Inter I;
    std::vector<Far> far;
    for (int k = 0; k < nsteps; ++k) {
        const uint64_t step1 = step0 + k + 1;
        baseline_step(mdl, X, step1, Y, I, far);
        const double rain = mdl.rain_of(step1);
#pragma omp parallel for schedule(dynamic, 1)
        for (int t = 0; t < (int)qs.size(); ++t) advance(mdl, qs[t], X, Y, I, far, rain);
        std::swap(X, Y);
    }
}

}  // namespace

extern "C" {

int hgo_fd_ref(int n, const float* settings, int period, uint64_t step0, int nsteps, const double* b0,
               const float* ks, const double* target, int m, const int* cells, const int* params, double eps,
               double* out) {
    if (n <= 0 || nsteps < 0 || m < 0) return -1;
    const size_t c = (size_t)n * n;
    for (int j = 0; j < m; ++j)
        if (cells[j] < 0 || (size_t)cells[j] >= c || (params[j] != 0 && params[j] != 1)) return -1;
    const Model mdl = make_model(n, settings, period, ks);
    if (mdl.p.Kspeed != 0.0) {  // talus slippage is not windowed: full forwards in parallel
        int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : bad)
        for (int j = 0; j < m; ++j) {
            const size_t cell = (size_t)cells[j];
            std::vector<double> bp(b0, b0 + c), bm(b0, b0 + c), fp(c), fm(c);
            std::vector<float> kp(ks, ks + c), km(ks, ks + c);
            double h;
            if (params[j] == 0) {
                kp[cell] = (float)((double)ks[cell] + eps);
                km[cell] = (float)((double)ks[cell] - eps);
                h = (double)kp[cell] - (double)km[cell];
            } else {
                bp[cell] += eps;
                bm[cell] -= eps;
                h = bp[cell] - bm[cell];
            }
            if (hgo_forward_ref(n, settings, period, step0, nsteps, bp.data(), kp.data(), fp.data()) ||
                hgo_forward_ref(n, settings, period, step0, nsteps, bm.data(), km.data(), fm.data()))
                bad += 1;
            double dl = 0;
            for (size_t i = 0; i < c; ++i) dl += (fp[i] - fm[i]) * (fp[i] + fm[i] - 2.0 * target[i]);
            out[j] = dl / (double)c / h;
        }
        return bad ? -1 : 0;
    }
    // 2j is the + side of pair j, 2j + 1 the - side
    std::vector<Perturbed> qs;
    std::vector<double> h(m);
    for (int j = 0; j < m; ++j) {
        qs.push_back(start(b0, ks, n, cells[j], params[j], eps));
        qs.push_back(start(b0, ks, n, cells[j], params[j], -eps));
        h[j] = params[j] == 0 ? (double)qs[2 * j].kval - (double)qs[2 * j + 1].kval
                              : qs[2 * j].b[0] - qs[2 * j + 1].b[0];
    }
    State X;
    run_windowed(mdl, b0, step0, nsteps, qs, X);
    for (int j = 0; j < m; ++j) {
        const Perturbed &qp = qs[2 * j], &qm = qs[2 * j + 1];
        Rect U = qp.R;
        U.add(qm.R.x0, qm.R.y0);
        U.add(qm.R.x1, qm.R.y1);
        double dl = 0;
        for (int y = U.y0; y <= U.y1; ++y)
            for (int x = U.x0; x <= U.x1; ++x) {
                const size_t i = (size_t)y * n + x;
                const double bp = qp.R.has(x, y) ? qp.b[qp.R.at(x, y)] : X.b[i];
                const double bm = qm.R.has(x, y) ? qm.b[qm.R.at(x, y)] : X.b[i];
                dl += (bp - bm) * (bp + bm - 2.0 * target[i]);
            }
        out[j] = dl / (double)c / h[j];
    }
    return 0;
}

// Final rock of one windowed perturbed forward (its own state on its
// rectangle, the baseline's elsewhere) and the rectangle's cell count: the
// test of hgo_fd_ref's windowing against full forwards of the same inputs.
int hgo_fd_ref_final(int n, const float* settings, int period, uint64_t step0, int nsteps, const double* b0,
                     const float* ks, int cell, int param, double delta, double* b_out, int* rect_cells) {
    const size_t c = (size_t)n * n;
    if (n <= 0 || nsteps < 0 || cell < 0 || (size_t)cell >= c || (param != 0 && param != 1)) return -1;
    const Model mdl = make_model(n, settings, period, ks);
    if (mdl.p.Kspeed != 0.0) return -1;
    std::vector<Perturbed> qs{start(b0, ks, n, cell, param, delta)};
    State X;
    run_windowed(mdl, b0, step0, nsteps, qs, X);
    const Perturbed& q = qs[0];
    for (size_t i = 0; i < c; ++i) {
        const int x = (int)(i % n), y = (int)(i / n);
        b_out[i] = q.R.has(x, y) ? q.b[q.R.at(x, y)] : X.b[i];
    }
    *rect_cells = q.R.w() * q.R.h();
    return 0;
}

}  // extern "C"
