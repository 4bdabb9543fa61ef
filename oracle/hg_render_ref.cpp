// CPU restatement of the terrain ray-marcher — TEST INFRASTRUCTURE ONLY
// (checks hg_render.cu).  Follows glsl/rendering.glsl in float, one rounding
// per GLSL operation (built without contraction):
//
//   main / to_world          :518-539     raymarch            :462-516
//   get_pixel_color          :393-460     get_water_color     :319-391
//   refractCameraRay         :304-317     get_terrain_color   :289-302
//   get_shade                :227-283     get_sky_color       :182-220
//   get_fog_color            :174-180     get_img_normal(_w)  :148-172
//   get_material_color       :115-146     fog_mix             :105-107
//   img_bilinear             glsl/img_interpolation.glsl:3-22
//
// pow and exp have no defined float result in GLSL; both sides evaluate them
// as exp2(y log2 x) with the same published series: log2 through
// ln m = 2 atanh((m - 1) / (m + 1)) on m in [sqrt(1/2), sqrt(2)) to s^9, and
// exp2 through the Taylor series of e^(f ln 2) to degree 7 on f in
// [-1/2, 1/2].  The view and perspective inverses are Gauss-Jordan with
// partial pivoting in double, rounded to float.
#include <cmath>
#include <cstdint>
#include <cstring>

namespace {

struct Vec {
    float x, y, z;
};
Vec mk(float x, float y, float z) { return Vec{x, y, z}; }
Vec operator+(Vec a, Vec b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
Vec operator-(Vec a, Vec b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
Vec operator*(Vec a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
Vec operator-(Vec a) { return mk(-a.x, -a.y, -a.z); }
float dot(Vec a, Vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
float length(Vec a) { return std::sqrt(dot(a, a)); }
Vec normalize(Vec a) {
    float l = length(a);
    return mk(a.x / l, a.y / l, a.z / l);
}
Vec cross(Vec a, Vec b) { return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
float fmin_(float x, float y) { return y < x ? y : x; }
float fmax_(float x, float y) { return x < y ? y : x; }
float clampf(float x, float lo, float hi) { return fmin_(fmax_(x, lo), hi); }
float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
Vec mixv(Vec a, Vec b, float t) { return mk(mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)); }
Vec reflect(Vec i, Vec n) { return i - n * (2.0f * dot(n, i)); }
float smoothstep(float e0, float e1, float x) {
    float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
float fractf(float x) { return x - std::floor(x); }
float bits_to_float(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
uint32_t float_to_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

float ex2(float x) {
    if (std::isnan(x)) return x;
    if (x >= 128.0f) return INFINITY;
    if (x < -150.0f) return 0.0f;
    float n = std::floor(x + 0.5f);
    float t = (x - n) * 0.693147180559945309f;
    const float c[8] = {1.0f / 5040.0f, 1.0f / 720.0f, 1.0f / 120.0f, 1.0f / 24.0f, 1.0f / 6.0f, 0.5f, 1.0f, 1.0f};
    float p = c[0];
    for (int k = 1; k < 8; ++k) p = p * t + c[k];
    int ni = (int)n, a = ni / 2, b = ni - a;
    return p * bits_to_float((uint32_t)(a + 127) << 23) * bits_to_float((uint32_t)(b + 127) << 23);
}

float lg2(float x) {
    int e = 0;
    if (x < 0x1p-126f) {
        x *= 0x1p23f;
        e = -23;
    }
    uint32_t u = float_to_bits(x);
    e += (int)((u >> 23) & 0xffu) - 127;
    float m = bits_to_float((u & 0x7fffffu) | 0x3f800000u);
    if (m > 1.41421356f) {
        m *= 0.5f;
        e += 1;
    }
    float s = (m - 1.0f) / (m + 1.0f), s2 = s * s;
    const float c[5] = {1.0f / 9.0f, 1.0f / 7.0f, 1.0f / 5.0f, 1.0f / 3.0f, 1.0f};
    float q = c[0];
    for (int k = 1; k < 5; ++k) q = q * s2 + c[k];
    return (float)e + 2.0f * s * q * 1.44269504088896341f;
}

float powf_(float x, float y) {
    if (!(x >= 0.0f)) return NAN;
    if (x == 0.0f) return y > 0.0f ? 0.0f : (y == 0.0f ? 1.0f : INFINITY);
    if (std::isinf(x)) return y > 0.0f ? x : (y == 0.0f ? 1.0f : 0.0f);
    return ex2(y * lg2(x));
}
float expf_(float x) { return ex2(x * 1.44269504088896341f); }

const float MAXD = 2048.0f;
const int MAXS = 1024;
enum { TOTAL = 3, TERRAIN = 4 };

struct Texel {
    float r, g, b, w;
};

struct World {
    int n;
    const float *rock, *dirt, *water, *s0, *s1;
    float max_height, prec;
    Vec light;
    Texel at(int x, int y) const {
        if (x < 0 || y < 0 || x >= n || y >= n) return Texel{0, 0, 0, 0};
        size_t i = (size_t)y * n + x;
        float r = rock[i], g = dirt ? dirt[i] : 0.0f, b = water[i];
        return Texel{r, g, b, r + g + b};
    }
    // img_bilinear of the heightmap (texel i = int(p), weight fract(p))
    Texel bil(float px, float py) const {
        if (!(px > -2.0f && px < (float)n + 1.0f && py > -2.0f && py < (float)n + 1.0f)) return Texel{0, 0, 0, 0};
        int ix = (int)px, iy = (int)py;
        float fx = fractf(px), fy = fractf(py);
        Texel a = at(ix, iy), b = at(ix + 1, iy), c = at(ix, iy + 1), d = at(ix + 1, iy + 1);
        auto m = [&](float va, float vb, float vc, float vd) { return mixf(mixf(va, vb, fx), mixf(vc, vd, fx), fy); };
        return Texel{m(a.r, b.r, c.r, d.r), m(a.g, b.g, c.g, d.g), m(a.b, b.b, c.b, d.b), m(a.w, b.w, c.w, d.w)};
    }
    void sed_bil(float px, float py, float& sr, float& sg) const {
        sr = sg = 0.0f;
        if (!(px > -2.0f && px < (float)n + 1.0f && py > -2.0f && py < (float)n + 1.0f)) return;
        int ix = (int)px, iy = (int)py;
        float fx = fractf(px), fy = fractf(py);
        auto t = [&](const float* f, int x, int y) {
            return (f && x >= 0 && y >= 0 && x < n && y < n) ? f[(size_t)y * n + x] : 0.0f;
        };
        auto m = [&](const float* f) {
            return mixf(mixf(t(f, ix, iy), t(f, ix + 1, iy), fx), mixf(t(f, ix, iy + 1), t(f, ix + 1, iy + 1), fx), fy);
        };
        sr = m(s0);
        sg = m(s1);
    }
};

struct Ray {
    Vec pos;
    float w, dist;
    Texel terr;
};

Ray raymarch(const World& W, Vec origin, Vec dir, float max_dst, int max_iter, int kind) {
    float dist = 0.001f, d_dist = 0.1f;
    if (kind == TERRAIN) {
        dist = 0.0f;
        d_dist = 0.1e-12f;
    }
    float min_sdf = 1.0f;
    Texel terr{0, 0, 0, 0};
    for (int i = 0; i < max_iter; ++i) {
        Vec sp = origin + dir * dist;
        terr = W.bil(sp.x, sp.z);
        float t_height = kind == TERRAIN ? terr.r + terr.g : terr.w;
        if ((sp.y > W.max_height && dir.y >= 0.0f) || (sp.y <= 0.0f && dir.y < 0.0f)) break;
        float d_height = sp.y - t_height;
        if (std::fabs(d_height) <= 0.05f) {
            Vec q = sp - dir * 0.05f;
            return Ray{q, 0.0f, dist - 0.05f, W.bil(q.x, q.z)};
        } else if (d_height < 0.0f) {
            return Ray{origin + dir * dist, min_sdf, dist, terr};
        }
        min_sdf = fmin_(min_sdf, 12.0f * d_dist / dist);
        if (dist > max_dst) return Ray{sp, min_sdf, max_dst, terr};
        d_dist = W.prec * d_height;
        dist += d_dist;
    }
    return Ray{origin + dir * max_dst, min_sdf, max_dst, terr};
}

float fog_mix(float f) { return clampf(f * f, 0.0f, 1.0f); }

struct Mat {
    Vec grass, rock, dirt;
};
const Mat AMBIENT{mk(0.00014f, 0.00084f, 0.00018f), mk(0.0008f, 0.0008f, 0.0008f), mk(0.00032f, 0.00030f, 0.0018f)};
const Mat DIFFUSE{mk(0.2068f, 0.279f, 0.01f) * 1.3f, mk(0.40f, 0.39f, 0.37f) * 1.3f,
                  mk(0.1968f, 0.169f, 0.03f) * 1.3f};
Mat diffuse_mat() {  // vec3(...) * 1.3 / 5 (grass), / 6 (rock, dirt)
    Vec g = DIFFUSE.grass, r = DIFFUSE.rock, d = DIFFUSE.dirt;
    return Mat{mk(g.x / 5.0f, g.y / 5.0f, g.z / 5.0f), mk(r.x / 6.0f, r.y / 6.0f, r.z / 6.0f),
               mk(d.x / 6.0f, d.y / 6.0f, d.z / 6.0f)};
}
const Vec SKY = mk(0.3f, 0.5f, 0.85f);

Vec material(const Ray& ray, Vec norm, const Mat& m) {
    float cos_a = dot(norm, mk(-0.0f, -1.0f, -0.0f));
    float dirt = smoothstep(0.0f, 1.0f, fmin_(1.0f, ray.terr.g));
    Vec col = m.rock;
    if (dirt > 0.0f) {
        if (cos_a < 0.75f) col = mixv(m.dirt, m.dirt * 0.4f, 1.0f - smoothstep(0.25f, 0.75f, cos_a));
        else if (cos_a < 0.95f) col = mixv(m.grass, m.dirt, 1.0f - smoothstep(0.85f, 0.95f, cos_a));
        else col = m.grass;
        col = mixv(m.rock, col, dirt);
    } else {
        col = mixv(m.rock, m.rock * 0.5f, 1.0f - smoothstep(0.0f, 0.65f, cos_a));
    }
    return col;
}

Vec normal_terrain(const World& W, float x, float z) {
    Texel r = W.bil(x + 1.0f, z + 0.0f), l = W.bil(x + -1.0f, z + 0.0f);
    Texel b = W.bil(x + 0.0f, z + -1.0f), t = W.bil(x + 0.0f, z + 1.0f);
    float dx = r.r + r.g - l.r - l.g;
    float dz = t.r + t.g - b.r - b.g;
    return normalize(cross(mk(2.0f, dx, 0.0f), mk(0.0f, dz, 2.0f)));
}

Vec normal_water(const World& W, float x, float z) {
    float dx = W.bil(x + 1.0f, z + 0.0f).w - W.bil(x + -1.0f, z + 0.0f).w;
    float dz = W.bil(x + 0.0f, z + 1.0f).w - W.bil(x + 0.0f, z + -1.0f).w;
    return normalize(cross(mk(2.0f, dx, 0.0f), mk(0.0f, dz, 2.0f)));
}

Vec fog(Vec col, float ray_dist, float sundot) {
    float fo = 1.0f - expf_(-powf_(0.15f * ray_dist / MAXD, 2.5f));
    Vec fco = mk(0.4f, 0.65f, 1.0f) * 0.65f + mk(1.0f, 0.8f, 0.5f) * 0.1f * powf_(sundot * 1.5f, 4.0f);
    return mixv(col, fco, fo);
}

Vec sky(Vec dir, float sundot) {
    float diry = dir.y;
    float dd = diry * diry * 0.37f;
    Vec col = mk(SKY.x - dd, SKY.y - dd, SKY.z - dd);
    col = mixv(col, mk(0.7f, 0.75f, 0.85f) * 0.85f, powf_(1.0f - fmax_(diry, 0.0f), 4.0f));
    col = col + mk(1.0f, 0.7f, 0.4f) * 0.25f * powf_(sundot, 5.0f);
    col = col + mk(1.0f, 0.8f, 0.6f) * 0.25f * powf_(sundot, 64.0f);
    col = col + mk(1.0f, 0.8f, 0.6f) * 0.2f * powf_(sundot, 512.0f);
    return mixv(col, mk(0.4f, 0.65f, 1.0f) * 0.68f, powf_(1.0f - fmax_(diry, 0.0f), 16.0f));
}

void shade(const World& W, const Ray& ray, Vec normal, bool is_water, Vec& rgb, float& w) {
    float shadow_diff = W.max_height - ray.pos.y;
    float shadow_scale = shadow_diff / -W.light.y;
    float shadow_max = length(W.light * shadow_scale);
    Ray shadow = raymarch(W, ray.pos, -W.light, shadow_max, MAXS / 2, TERRAIN);
    float amb_factor = clampf(0.5f + 0.5f * -normal.y, 0.0f, 1.0f);
    Vec ambient, diffuse;
    if (is_water) {
        ambient = SKY * 0.005f;
        diffuse = mk(0.108f, 0.187f, 0.288f) * 0.1f;
    } else {
        ambient = material(ray, -normal, AMBIENT);
        diffuse = material(ray, normal, diffuse_mat());
    }
    ambient = ambient + (diffuse + SKY * 0.01f) * (amb_factor * 0.20f);
    rgb = ambient;
    w = 0.04f;
    if (shadow.dist >= shadow_max) {
        float lambrt = fmax_(dot(W.light, normal), 0.0f);
        rgb = rgb + diffuse * lambrt * shadow.w;
        w = shadow.w;
    }
}

Vec terrain_col(const World& W, const Ray& ray, Vec dir, float sundot) {
    Vec normal = normal_terrain(W, ray.pos.x, ray.pos.z);
    Vec col;
    float w;
    shade(W, ray, normal, false, col, w);
    col = fog(col, ray.dist, sundot);
    return mixv(col, sky(dir, sundot), fog_mix(ray.dist / MAXD));
}

Vec refract_cam(Vec n, Vec d, float eta) {
    float cos_t = dot(-n, d);
    float sin_t2 = 1.0f - cos_t * cos_t;
    float sin_p2 = eta * eta * sin_t2;
    if (sin_p2 > 1.0f) return reflect(d, n);
    float cos_p = std::sqrt(1.0f - sin_p2);
    return d * eta + n * (eta * cos_t - cos_p);
}

Vec water_col(const World& W, const Ray& w_ray, Vec dir, float sundot) {
    Vec w_norm = normal_water(W, w_ray.pos.x, w_ray.pos.z);
    Vec rdir = refract_cam(w_norm, dir, 1.0f / 1.3f);
    Ray t_ray = raymarch(W, w_ray.pos, -rdir, MAXD / 8.0f, MAXS / 4, TERRAIN);
    float water_vol = t_ray.dist;
    t_ray.dist += w_ray.dist;
    Vec t_shad = terrain_col(W, t_ray, dir, sundot);
    Vec w_refl = reflect(dir, w_norm);
    Ray wr = raymarch(W, w_ray.pos, w_refl, MAXD, MAXS, TERRAIN);
    Vec ws_rgb;
    float ws_w;
    shade(W, w_ray, w_norm, true, ws_rgb, ws_w);
    Vec col = ws_rgb;
    float refl_sundot = clampf(dot(w_refl, -W.light), 0.0f, 1.0f);
    Vec sky_r = sky(w_refl, refl_sundot);
    float cos_theta = dot(dir, w_norm);
    float fresnel = fmax_(powf_(1.0f - cos_theta, 2.0f), 0.06f);
    if (wr.dist >= MAXD) {
        col = mixv(t_shad, col, fmin_(1.0f, water_vol / 2.0f));
        col = mixv(col, sky_r, fresnel);
        col = mixv(ws_rgb, col, ws_w);
    } else {
        wr.dist += w_ray.dist;
        col = mixv(t_shad, col, fmin_(1.0f, water_vol / 2.0f));
        col = mixv(col, terrain_col(W, wr, w_refl, refl_sundot), ws_w);
        col = mixv(t_shad, col, fresnel);
        col = mixv(col, sky_r, fog_mix(wr.dist / MAXD));
    }
    return col;
}

bool inverse4(const float* m, float* out) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            a[r][c] = m[c * 4 + r];
            a[r][4 + c] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[p][c])) p = r;
        if (a[p][c] == 0.0 || !std::isfinite(a[p][c])) return false;
        if (p != c)
            for (int k = 0; k < 8; ++k) {
                double t = a[p][k];
                a[p][k] = a[c][k];
                a[c][k] = t;
            }
        double inv = 1.0 / a[c][c];
        for (int k = 0; k < 8; ++k) a[c][k] *= inv;
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            double f = a[r][c];
            if (f == 0.0) continue;
            for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[c * 4 + r] = (float)a[r][4 + c];
    return true;
}

void mulv(const float* m, const float v[4], float r[4]) {
    for (int i = 0; i < 4; ++i) r[i] = m[i] * v[0] + m[4 + i] * v[1] + m[8 + i] * v[2] + m[12 + i] * v[3];
}

void to_world(const float* ip, const float* iv, const float c[4], float out[4]) {
    float t[4];
    mulv(ip, c, t);
    float w = t[3];
    float u[4] = {t[0] / w, t[1] / w, t[2] / w, t[3] / w};
    mulv(iv, u, out);
}

unsigned char unorm8(float f) {
    f = f > 0.0f ? (f < 1.0f ? f : 1.0f) : 0.0f;
    return (unsigned char)std::floor(f * 255.0f + 0.5f);
}

}  // namespace

extern "C" {

// Camera as hg_camera (include/hydrogen.h).
struct OracleCamera {
    float view[16], perspective[16], pos[3], prec;
    int32_t draw_water, display_sediment;
    float sediment_max_cap;
    int32_t low_res_div3;
};

// Renders width x height RGBA8 pixels (row 0 first) and the float colour;
// dirt / s1 may be NULL (one-layer world).  Returns -1 for singular matrices.
int hgo_render(const float* rock, const float* dirt, const float* water, const float* s0, const float* s1, int n,
               float max_height, int hmap_dim_x, const OracleCamera* cam, int width, int height, uint8_t* rgba,
               float* rgb) {
    float ip[16], iv[16];
    if (!inverse4(cam->perspective, ip) || !inverse4(cam->view, iv)) return -1;
    World W{n, rock, dirt, water, s0, s1, max_height, cam->prec, normalize(mk(0.0f, -0.7f, 1.0f))};
    const bool low = cam->low_res_div3 != 0;
    const int wd = low ? width / 3 : width, hd = low ? height / 3 : height;
    const float alpha = low ? (float)hmap_dim_x : 0.0f;
    if (low) {
        std::memset(rgba, 0, (size_t)width * height * 4);
        if (rgb) std::memset(rgb, 0, (size_t)width * height * 3 * sizeof(float));
    }
    const Vec pos = mk(cam->pos[0], cam->pos[1], cam->pos[2]);
#pragma omp parallel for schedule(dynamic, 1)
    for (int py = 0; py < hd; ++py)
        for (int px = 0; px < wd; ++px) {
            float ux = (float)px / (float)wd, uy = (float)py / (float)hd;
            float c0[4] = {0.0f, 0.0f, -1.0f, 1.0f}, c1[4] = {2.0f * ux - 1.0f, 2.0f * uy - 1.0f, 1.0f, 1.0f};
            float rs[4], re[4];
            to_world(ip, iv, c0, rs);
            to_world(ip, iv, c1, re);
            Vec dir = normalize(mk(re[0] - rs[0], re[1] - rs[1], re[2] - rs[2]));
            Ray ray = raymarch(W, pos, dir, MAXD, MAXS, TOTAL);
            float sundot = clampf(dot(dir, -W.light), 0.0f, 1.0f);
            float pxz = ray.pos.x * 1.0f, pzz = ray.pos.z * 1.0f;
            float water_h = fmin_(1.0f, smoothstep(1e-4f, 1.0f, ray.terr.b));
            Vec color;
            if (pxz < 0.0f || pxz >= (float)n || pzz < 0.0f || pzz >= (float)n) {
                color = sky(dir, sundot);
            } else if (ray.dist >= MAXD) {
                color = sky(dir, sundot);
            } else if (water_h > 1e-12f && cam->draw_water) {
                Vec wc = fog(water_col(W, ray, dir, sundot), ray.dist, sundot);
                color = mixv(wc, sky(dir, sundot), fog_mix(ray.dist / MAXD));
            } else {
                color = terrain_col(W, ray, dir, sundot);
            }
            if (cam->display_sediment) {
                float sr, sg;
                W.sed_bil(ray.pos.x, ray.pos.z, sr, sg);
                color = mixv(color, mk(1.0f, 0.0f, 0.0f), fmin_(1.0f, sr / cam->sediment_max_cap));
                color = mixv(color, mk(0.0f, 1.0f, 0.0f), fmin_(1.0f, sg / cam->sediment_max_cap));
            }
            const float gam = 1.0f / 2.2f;
            color = mk(powf_(color.x, gam), powf_(color.y, gam), powf_(color.z, gam));
            const int rep = low ? 3 : 1;
            for (int oy = 0; oy < rep; ++oy)
                for (int ox = 0; ox < rep; ++ox) {
                    size_t o = (size_t)(py * rep + oy) * width + (px * rep + ox);
                    rgba[4 * o + 0] = unorm8(color.x);
                    rgba[4 * o + 1] = unorm8(color.y);
                    rgba[4 * o + 2] = unorm8(color.z);
                    rgba[4 * o + 3] = unorm8(alpha);
                    if (rgb) {
                        rgb[3 * o + 0] = color.x;
                        rgb[3 * o + 1] = color.y;
                        rgb[3 * o + 2] = color.z;
                    }
                }
        }
    return 0;
}

// the ray-marcher's pow / exp2 / log2, for accuracy tests against libm
float hgo_render_pow(float x, float y) { return powf_(x, y); }
float hgo_render_exp2(float x) { return ex2(x); }
float hgo_render_log2(float x) { return lg2(x); }

}  // extern "C"
