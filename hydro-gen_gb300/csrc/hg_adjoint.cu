// Reverse-mode adjoint of the grid step without thermal erosion.
//
// One reversed step works on the step's input state X (restored from a
// checkpoint and recomputed) and the adjoint A of its outputs:
//   k_adj_recompute  rain, flux and erosion of every cell (the forward cell
//                    code of hg_device.cuh, so the intermediates are the
//                    forward's own bits): water after rain, u, v, d1+d2, d2,
//                    eroded rock and sediment
//   k_adj_sediment   semi-Lagrangian gather reversed: each cell scatters its
//                    sediment adjoint to its four taps (atomicAdd: the taps
//                    of a back-trace are data dependent), and the velocity
//                    adjoint of the back-trace point
//   k_adj_erosion    dissolve/deposit/exhaustion branch reversed; the
//                    terrain normal's neighbour terms become per-cell
//                    packets; per-cell Ks gradient accumulated
//   k_adj_flux       outflow, scaling, water update and velocity reversed;
//                    neighbour terms become per-cell packets
//   k_adj_gather     every cell sums its own terms and its neighbours'
//                    packets into the input adjoint (deterministic order)
// Subgradients: max(0, x) and min(1, q) pass the derivative of the taken
// argument (ties take the constant side), clamps pass 0 when clamped,
// dissolve/deposit/exhaustion use the taken branch, floor() is locally
// constant.  The formulas follow the shaders cited in hg_device.cuh.
#include "hg_internal.h"

namespace hg {

namespace {

constexpr int BX = 32, BY = 8;
__device__ __forceinline__ size_t at(int n, int x, int y) { return (size_t)y * n + x; }

// water after this step's rain
__global__ void k_adj_rain(StepConsts c, RainStep r, const float* __restrict__ d, float* __restrict__ dr) {
    int x0 = (blockIdx.x * blockDim.x + threadIdx.x) * 4;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x0 >= c.n || y >= c.n) return;
    size_t i = at(c.n, x0, y);
    float4 v = *reinterpret_cast<const float4*>(d + i);
    if (r.active) {
        uint32_t w[4] = {0, 0, 0, 0};
        if (r.bernoulli) rain_words4(r, x0, y, w);
        v.x += rain_incr(r, w[0]);
        v.y += rain_incr(r, w[1]);
        v.z += rain_incr(r, w[2]);
        v.w += rain_incr(r, w[3]);
    }
    *reinterpret_cast<float4*>(dr + i) = v;
}

__global__ void k_adj_recompute(StepConsts c, AdjFields X, AdjTemps T) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y >= n) return;
    size_t i = at(n, x, y);
    auto w = [&](int xx, int yy) -> float {
        if (xx < 0 || xx >= n || yy < 0 || yy >= n) return FAR_HEIGHT;
        size_t j = at(n, xx, yy);
        return X.b[j] + T.dr[j];
    };
    float d1 = T.dr[i];
    float inl = x > 0 ? X.f[1][i - 1] : 0.0f;
    float inr = x < n - 1 ? X.f[0][i + 1] : 0.0f;
    float int_ = y < n - 1 ? X.f[3][i + n] : 0.0f;
    float inb = y > 0 ? X.f[2][i - n] : 0.0f;
    FluxOut o = cell_flux(c, x, y, X.b[i] + d1, d1, X.f[0][i], X.f[1][i], X.f[2][i], X.f[3][i], w(x - 1, y),
                          w(x + 1, y), w(x, y + 1), w(x, y - 1), inl, inr, int_, inb);
    float b = X.b[i], s = X.s[i];
    float br = x < n - 1 ? X.b[i + 1] : 0.0f, bl = x > 0 ? X.b[i - 1] : 0.0f;
    float bb = y > 0 ? X.b[i - n] : 0.0f, bt = y < n - 1 ? X.b[i + n] : 0.0f;
    float Kls0 = c.ks_field ? c.dt * c.ks_field[i] : c.Kls0;
    cell_erosion(c, Kls0, o.u, o.v, o.vz, b, s, br, bl, bb, bt);
    T.u[i] = o.u;
    T.v[i] = o.v;
    T.vz[i] = o.vz;
    T.d2[i] = o.d2;
    T.be[i] = b;
    T.se[i] = s;
}

__global__ void k_adj_sediment(StepConsts c, AdjFields A, AdjTemps T, AdjWork W) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y >= n) return;
    size_t i = at(n, x, y);
    W.dd2[i] = A.d[i] * c.evap;
    const float a = A.s[i];
    const float maxc = (float)(n - 1);
    float rx = (float)x - T.u[i] * c.dt, ry = (float)y - T.v[i] * c.dt;
    float px = gclamp(rx, 0.0f, maxc), py = gclamp(ry, 0.0f, maxc);
    int ix = min(max((int)px, 0), n - 1), iy = min(max((int)py, 0), n - 1);
    float fx = px - floorf(px), fy = py - floorf(py);
    auto S = [&](int xx, int yy) -> float {
        return (xx < n && yy < n) ? T.se[at(n, xx, yy)] : 0.0f;
    };
    auto add = [&](int xx, int yy, float v) {
        if (xx < n && yy < n && v != 0.0f) atomicAdd(W.dse + at(n, xx, yy), v);
    };
    add(ix, iy, a * (1.0f - fx) * (1.0f - fy));
    add(ix + 1, iy, a * fx * (1.0f - fy));
    add(ix, iy + 1, a * (1.0f - fx) * fy);
    add(ix + 1, iy + 1, a * fx * fy);
    float s00 = S(ix, iy), s10 = S(ix + 1, iy), s01 = S(ix, iy + 1), s11 = S(ix + 1, iy + 1);
    float dfx = (s10 - s00) * (1.0f - fy) + (s11 - s01) * fy;
    float dfy = (s01 * (1.0f - fx) + s11 * fx) - (s00 * (1.0f - fx) + s10 * fx);
    W.du[i] = (rx > 0.0f && rx < maxc) ? a * dfx * (-c.dt) : 0.0f;
    W.dv[i] = (ry > 0.0f && ry < maxc) ? a * dfy * (-c.dt) : 0.0f;
}

__global__ void k_adj_erosion(StepConsts c, AdjFields X, AdjFields A, AdjTemps T, AdjWork W, float* __restrict__ dks) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y >= n) return;
    size_t i = at(n, x, y);
    auto B = [&](int xx, int yy) -> float {
        return (xx < 0 || xx >= n || yy < 0 || yy >= n) ? 0.0f : X.b[at(n, xx, yy)];
    };
    float u = T.u[i], v = T.v[i], vz = T.vz[i];
    float len = sqrtf(u * u + v * v), ero = len, dero_dlen = 1.0f, dero_dvz = 0.0f;
    if (vz < 1e-3f) {
        float dd = gmax(5e-4f, vz);
        float tr = (dd - 1e-3f) / (5e-4f - 1e-3f);
        float t = gclamp(tr, 0.0f, 1.0f);
        float sm = t * t * (3.0f - 2.0f * t);
        ero = len * (1.0f - sm);
        dero_dlen = 1.0f - sm;
        if (vz > 5e-4f && tr > 0.0f && tr < 1.0f) dero_dvz = -len * 6.0f * t * (1.0f - t) / (5e-4f - 1e-3f);
    }
    float dx = B(x + 1, y) - B(x - 1, y), dz = B(x, y + 1) - B(x, y - 1);
    float L3 = sqrtf(4.0f * dx * dx + 16.0f + 4.0f * dz * dz);
    float ny = -4.0f / L3;
    float sin_a = sqrtf(1.0f - ny * ny);
    float sa = gmax(0.02f, sin_a);
    float craw = c.Kc * sa * ero;
    float cc = gmax(0.0f, craw);
    float Ks_i = c.ks_field ? c.ks_field[i] : c.Ks0;
    float Kls = c.dt * Ks_i, Kld = c.Kld0, b = X.b[i], s = X.s[i];
    float ab = A.b[i], as = W.dse[i];
    float gb, gs, gc = 0.0f, gK = 0.0f;
    if (cc > s) {
        float del = Kls * (cc - s);
        if (b - del < 0.0f) {  // rock exhausted: b' = 0, s' = s + b
            gb = as;
            gs = as;
        } else {
            gb = ab;
            gs = ab * Kls + as * (1.0f - Kls);
            gc = (as - ab) * Kls;
            gK = (as - ab) * (cc - s);
        }
    } else {
        gb = ab;
        gs = ab * Kld + as * (1.0f - Kld);
        gc = (as - ab) * Kld;
    }
    dks[i] += gK * c.dt;
    W.rb[i] = gb;
    W.rs[i] = gs;
    float pdx = 0.0f, pdz = 0.0f, du = 0.0f, dv = 0.0f, dvz = 0.0f;
    if (craw > 0.0f) {
        float gsa = gc * c.Kc * ero, gero = gc * c.Kc * sa;
        if (sin_a > 0.02f) {
            float gny = gsa * (-ny / sin_a);
            float gL3 = gny * (4.0f / (L3 * L3));
            pdx = gL3 * 4.0f * dx / L3;
            pdz = gL3 * 4.0f * dz / L3;
        }
        float glen = gero * dero_dlen;
        dvz = gero * dero_dvz;
        if (len > 0.0f) {
            du = glen * u / len;
            dv = glen * v / len;
        }
    }
    W.pdx[i] = pdx;
    W.pdz[i] = pdz;
    W.du[i] += du;
    W.dv[i] += dv;
    W.dvz[i] = dvz;
}

__global__ void k_adj_flux(StepConsts c, AdjFields X, AdjFields A, AdjTemps T, AdjWork W) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = c.n;
    if (x >= n || y >= n) return;
    size_t i = at(n, x, y);
    const int ox[4] = {-1, 1, 0, 0}, oy[4] = {0, 0, 1, -1};
    auto w = [&](int xx, int yy) -> float {
        if (xx < 0 || xx >= n || yy < 0 || yy >= n) return FAR_HEIGHT;
        size_t j = at(n, xx, yy);
        return X.b[j] + T.dr[j];
    };
    const float d1 = T.dr[i], wc = X.b[i] + d1;
    float ft[4], g[4];
    bool live[4];
    for (int k = 0; k < 4; ++k) {
        ft[k] = c.EK * X.f[k][i] + c.dt * (c.G * (wc - w(x + ox[k], y + oy[k])));
        g[k] = gmax(0.0f, ft[k]);
        live[k] = ft[k] > 0.0f;
    }
    if (x <= 0) { g[0] = 0.0f; live[0] = false; } else if (x >= n - 1) { g[1] = 0.0f; live[1] = false; }
    if (y <= 0) { g[3] = 0.0f; live[3] = false; } else if (y >= n - 1) { g[2] = 0.0f; live[2] = false; }
    float inl = x > 0 ? X.f[1][i - 1] : 0.0f, inr = x < n - 1 ? X.f[0][i + 1] : 0.0f;
    float it = y < n - 1 ? X.f[3][i + n] : 0.0f, ib = y > 0 ? X.f[2][i - n] : 0.0f;
    float sum_in = inl + inr + it + ib;
    float sum_out = g[0] + g[1] + g[2] + g[3];
    float den = sum_out * c.dt;
    bool scaled = !(d1 >= den) && (d1 / den) < 1.0f;  // K = d1/den (else K = 1)
    float K = scaled ? d1 / den : 1.0f;
    float arg = d1 + c.dt * (sum_in - sum_out * K);
    float vz = T.vz[i], u = T.u[i], v = T.v[i];
    float gvz = W.dvz[i], gin[4] = {0, 0, 0, 0}, gfown[4] = {0, 0, 0, 0};
    if (vz > 0.0f) {
        float du = W.du[i] / vz, dv = W.dv[i] / vz;
        gin[0] += du; gin[1] -= du;
        gfown[0] -= du; gfown[1] += du;
        gin[3] += dv; gin[2] -= dv;
        gfown[3] -= dv; gfown[2] += dv;
        gvz -= (W.du[i] * u + W.dv[i] * v) / vz;
    }
    float gd1 = gvz, gd2 = gvz + W.dd2[i];
    float garg = arg > 0.0f ? gd2 : 0.0f;
    gd1 += garg;
    float gsum_in = c.dt * garg, gsum_outK = -c.dt * garg;
    for (int k = 0; k < 4; ++k) gin[k] += gsum_in;
    float gK = gsum_outK * sum_out, gsum_out = gsum_outK * K;
    for (int k = 0; k < 4; ++k) gK += A.f[k][i] * g[k];
    float gg[4];
    for (int k = 0; k < 4; ++k) gg[k] = A.f[k][i] * K + gsum_out;
    if (scaled) {
        gd1 += gK / den;
        float gden = -gK * d1 / (den * den);
        for (int k = 0; k < 4; ++k) gg[k] += gden * c.dt;
    }
    float gw = 0.0f;
    for (int k = 0; k < 4; ++k) {
        float gdh = 0.0f;
        if (live[k]) {
            gfown[k] += c.EK * gg[k];
            gdh = c.dt * c.G * gg[k];
            gw += gdh;
        }
        W.pdh[k][i] = gdh;
        W.pin[k][i] = gin[k];
        W.fown[k][i] = gfown[k];
    }
    W.wbar[i] = gw;
    W.gd1[i] = gd1;
}

__global__ void k_adj_gather(int n, AdjWork W, AdjFields R) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= n || y >= n) return;
    size_t i = at(n, x, y);
    // w = rock + water: a neighbour's height difference toward this cell
    // (its direction opposite to ours) enters with a minus sign
    float nbw = 0.0f;
    if (x > 0) nbw += W.pdh[1][i - 1];      // left neighbour's R
    if (x < n - 1) nbw += W.pdh[0][i + 1];  // right neighbour's L
    if (y < n - 1) nbw += W.pdh[3][i + n];  // top neighbour's B
    if (y > 0) nbw += W.pdh[2][i - n];      // bottom neighbour's T
    float nrm = 0.0f;  // terrain-normal terms of the neighbours
    if (x > 0) nrm += W.pdx[i - 1];
    if (x < n - 1) nrm -= W.pdx[i + 1];
    if (y > 0) nrm += W.pdz[i - n];
    if (y < n - 1) nrm -= W.pdz[i + n];
    R.b[i] = W.rb[i] + W.wbar[i] - nbw + nrm;
    R.d[i] = W.wbar[i] + W.gd1[i] - nbw;
    R.s[i] = W.rs[i];
    R.f[0][i] = W.fown[0][i] + (x > 0 ? W.pin[1][i - 1] : 0.0f);      // left neighbour's inflow from me
    R.f[1][i] = W.fown[1][i] + (x < n - 1 ? W.pin[0][i + 1] : 0.0f);  // right neighbour's inflow from me
    R.f[2][i] = W.fown[2][i] + (y < n - 1 ? W.pin[3][i + n] : 0.0f);  // top neighbour's inflow from me
    R.f[3][i] = W.fown[3][i] + (y > 0 ? W.pin[2][i - n] : 0.0f);      // bottom neighbour's inflow from me
}

// d(mean((rock - target)^2))/d rock, and the loss partials
__global__ void k_mse_grad(const float* __restrict__ b, const float* __restrict__ target, size_t count,
                           float* __restrict__ grad, double* __restrict__ part) {
    __shared__ double sh[256 / 32];
    double acc = 0.0;
    const double inv = 1.0 / (double)count;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        float e = b[i] - target[i];
        acc += (double)e * (double)e;
        if (grad) grad[i] = (float)(2.0 * (double)e * inv);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
        part[blockIdx.x] = t * inv;
    }
}

__global__ void k_sum_parts(const double* __restrict__ part, int nparts, double* __restrict__ out) {
    if (threadIdx.x != 0) return;
    double t = 0.0;
    for (int k = 0; k < nparts; ++k) t += part[k];
    *out = t;
}

dim3 grid_for(int n) { return dim3((n + BX - 1) / BX, (n + BY - 1) / BY); }

}  // namespace

void launch_adjoint_step(const StepConsts& c, const RainStep& r, const AdjFields& X, const AdjFields& A,
                         const AdjFields& R, const AdjTemps& T, const AdjWork& W, float* dks, cudaStream_t st) {
    const int n = c.n;
    dim3 blk(BX, BY), g = grid_for(n), g4((n / 4 + BX - 1) / BX, (n + BY - 1) / BY);
    k_adj_rain<<<g4, blk, 0, st>>>(c, r, X.d, T.dr);
    k_adj_recompute<<<g, blk, 0, st>>>(c, X, T);
    cudaMemsetAsync(W.dse, 0, (size_t)n * n * sizeof(float), st);
    k_adj_sediment<<<g, blk, 0, st>>>(c, A, T, W);
    k_adj_erosion<<<g, blk, 0, st>>>(c, X, A, T, W, dks);
    k_adj_flux<<<g, blk, 0, st>>>(c, X, A, T, W);
    k_adj_gather<<<g, blk, 0, st>>>(n, W, R);
    count_launch(6);
}

void launch_mse(const float* b, const float* target, size_t count, float* grad, double* part, int nparts,
                double* out, cudaStream_t st) {
    k_mse_grad<<<nparts, 256, 0, st>>>(b, target, count, grad, part);
    k_sum_parts<<<1, 32, 0, st>>>(part, nparts, out);
    count_launch(2);
}

}  // namespace hg
