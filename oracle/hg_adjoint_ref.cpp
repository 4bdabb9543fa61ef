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

    void step(const State& X, uint64_t step1, State& Y, Inter& I) const {
        const size_t c = (size_t)n * n;
        Y.init(c);
        I.dr.assign(c, 0); I.u.assign(c, 0); I.v.assign(c, 0); I.vz.assign(c, 0); I.d2.assign(c, 0);
        I.be.assign(c, 0); I.se.assign(c, 0);
        const bool rains = p.period > 0 && step1 % (uint64_t)p.period == 0;
        for (size_t i = 0; i < c; ++i) I.dr[i] = X.d[i] + (rains ? p.amount : 0.0);
        auto w = [&](int x, int y) { return in(x, y) ? X.b[id(x, y)] + I.dr[id(x, y)] : FAR; };
        auto F = [&](int k, int x, int y) { return in(x, y) ? X.f[k][id(x, y)] : 0.0; };
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                size_t i = id(x, y);
                double wc = w(x, y), d1 = I.dr[i];
                const int ox[4] = {-1, 1, 0, 0}, oy[4] = {0, 0, 1, -1};
                double g[4];
                for (int k = 0; k < 4; ++k) {
                    double ft = p.EK * X.f[k][i] + p.dt * (p.G * (wc - w(x + ox[k], y + oy[k])));
                    g[k] = gmax(0.0, ft);
                }
                if (x <= 0) g[0] = 0; else if (x >= n - 1) g[1] = 0;
                if (y <= 0) g[3] = 0; else if (y >= n - 1) g[2] = 0;
                double inl = F(1, x - 1, y), inr = F(0, x + 1, y), it = F(3, x, y + 1), ib = F(2, x, y - 1);
                double sum_in = inl + inr + it + ib;
                double sum_out = g[0] + g[1] + g[2] + g[3];
                double K = gmin(1.0, d1 / (sum_out * p.dt));
                for (int k = 0; k < 4; ++k) Y.f[k][i] = g[k] * K;
                double d2 = gmax(0.0, d1 + p.dt * (sum_in - sum_out * K));
                double vz = d1 + d2;
                double u = 0, v = 0;
                if (vz > 0) {
                    u = (inl - X.f[0][i] + X.f[1][i] - inr) / vz;
                    v = (ib - X.f[3][i] + X.f[2][i] - it) / vz;
                }
                I.u[i] = u; I.v[i] = v; I.vz[i] = vz; I.d2[i] = d2;
            }
        // erosion
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                size_t i = id(x, y);
                auto B = [&](int xx, int yy) { return in(xx, yy) ? X.b[id(xx, yy)] : 0.0; };
                double u = I.u[i], v = I.v[i], vz = I.vz[i];
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
                double Kls = p.dt * (double)ks[i], b = X.b[i], s = X.s[i];
                if (cc > s) {
                    double del = Kls * (cc - s);
                    b -= del; s += del;
                    if (b < 0) { s += b; b = 0; }
                } else {
                    double del = (p.dt * p.Kd0) * (s - cc);
                    b += del; s -= del;
                }
                I.be[i] = b; I.se[i] = s;
            }
        // sediment transport + evaporation
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                size_t i = id(x, y);
                double px = gmin(gmax(x - I.u[i] * p.dt, 0.0), (double)(n - 1));
                double py = gmin(gmax(y - I.v[i] * p.dt, 0.0), (double)(n - 1));
                int ix = (int)px, iy = (int)py;
                double fx = px - std::floor(px), fy = py - std::floor(py);
                auto S = [&](int xx, int yy) { return in(xx, yy) ? I.se[id(xx, yy)] : 0.0; };
                double v1 = S(ix, iy) * (1 - fx) + S(ix + 1, iy) * fx;
                double v2 = S(ix, iy + 1) * (1 - fx) + S(ix + 1, iy + 1) * fx;
                Y.s[i] = v1 * (1 - fy) + v2 * fy;
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
    for (int k = 0; k < nsteps; ++k) {
        Inter I;
        m.step(X, step0 + k + 1, Y, I);
        X = Y;
    }
    for (size_t i = 0; i < c; ++i) b_out[i] = X.b[i];
    return 0;
}

}  // extern "C"
