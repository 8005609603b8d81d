/*
 * CPU ORACLE for the pyvr ray-marching path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this file's library, and only to check or time against; nothing in the
 * pyvr_gb300 package calls it.
 *
 * A single-precision restatement, line by line, of the reference fragment
 * shader pyvr/shaders/volume.frag.glsl:25-121 (with the vertex stage
 * pyvr/shaders/volume.vert.glsl:8), plus the GL state the reference sets up
 * around it:
 *   - 3D textures, LINEAR filtering, CLAMP_TO_EDGE, size = data.shape
 *     (pyvr/moderngl_renderer/manager.py:95-101, 123-129);
 *   - the RGBA LUT as a (size x 1) LINEAR/CLAMP texture (manager.py:178-181);
 *   - clear to 0 and blend SRC_ALPHA / ONE_MINUS_SRC_ALPHA on all four
 *     channels into an RGBA8 target (manager.py:29-31, 212-220);
 *   - read-back bottom row first (manager.py:228-230).
 * The camera/light uniforms are taken exactly as the reference renderer
 * sends them (renderer.py:148-172, 303-316): raw float32 bytes of the
 * numpy matrices, read by GL column-major.
 *
 * Rounding is pinned so that the result is a deterministic function of the
 * inputs (GLSL leaves these choices to the driver):
 *   - no contraction: every a*b+c is a rounded product then a rounded sum,
 *     except the texture-filter lerps, which are lerp(a,b,t) = fmaf(t, b-a, a);
 *   - matrix inverses in double, rounded to float once;
 *   - division by the box extent is a multiply by its float reciprocal;
 *   - step/reference_step_size is folded into one float factor;
 *   - exp is oracle_expf below (Cody-Waite reduction + degree-7 Taylor);
 *   - normalize(v) = v * rsqrt(dot(v,v)) with the reciprocal square root
 *     rounded once to float, computed as (float)(1.0 / sqrt((double)x))
 *     (the double quotient is rounded to the same float as the exact value
 *     for every positive float input: checked exhaustively against the
 *     GPU's correctly rounded __frsqrt_rn); a zero vector shades with a
 *     diffuse term of 0 (what max(dot(NaN, L), 0) gives under IEEE maxNum);
 *   - UNORM8 store = rintf(x * 255) of the clamped blended value.
 * Build with -ffp-contract=off.  No image-level golden data exists for this
 * path in the reference (its renderer tests mock GL), so image parity is
 * anchored on this restatement and the known-answer tests in tests/.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_U8 0
#define ORACLE_F16 1
#define ORACLE_F32 2

typedef struct {
    int width, height;
    float view[16];      /* numpy row-major bytes of Camera.get_view_matrix()        */
    float proj[16];      /* numpy row-major bytes of Camera.get_projection_matrix()  */
    float cam_pos[3];
    const void *volume;  /* shape (D,H,W) C-order                                    */
    int dtype;           /* ORACLE_U8 / ORACLE_F16 / ORACLE_F32                      */
    int dims[3];         /* D, H, W                                                  */
    float value_scale;   /* stored value -> density multiplier (1 = reference)       */
    const float *normals;/* (D,H,W,3) float32 or NULL                                */
    float bmin[3], bmax[3];
    const float *lut;    /* (lut_size, 4) float32 RGBA                               */
    int lut_size;
    float step_size, reference_step_size;
    int max_steps;
    float light_pos[3], light_target[3];
    float ambient, diffuse;
} OracleScene;

/* ---- helpers --------------------------------------------------------------*/

float oracle_expf(float x) {
    /* exp(x) = 2^k * exp(r), k = rint(x / ln2), r = x - k ln2 with ln2 split
     * into 0.693359375 (exact in 9 bits) + -2.12194440e-4 (Cody & Waite),
     * exp(r) by Taylor to r^7 for |r| <= ln2/2. Below -87.3 flushes to 0. */
    if (x != x) return x;
    if (x > 88.72283f) return INFINITY;
    if (x < -87.33654f) return 0.0f;
    float kf = rintf(x * 1.44269504f);
    float r = fmaf(kf, -0.693359375f, x);
    r = fmaf(kf, 2.12194440e-4f, r);
    float p = 1.98412698e-4f;            /* 1/7! */
    p = fmaf(p, r, 1.38888889e-3f);      /* 1/6! */
    p = fmaf(p, r, 8.33333333e-3f);      /* 1/5! */
    p = fmaf(p, r, 4.16666667e-2f);      /* 1/4! */
    p = fmaf(p, r, 1.66666667e-1f);      /* 1/3! */
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    int k = (int)kf;                     /* -126 .. 128 */
    int k1 = k > 0 ? k / 2 : 0;          /* split 2^k for k = 128 */
    int k2 = k - k1;
    union { uint32_t u; float f; } s1, s2;
    s1.u = (uint32_t)(k1 + 127) << 23;
    s2.u = (uint32_t)(k2 + 127) << 23;
    return (p * s1.f) * s2.f;
}

static float half_to_float(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1f, m = h & 0x3ffu;
    union { uint32_t u; float f; } o;
    if (e == 0) {
        if (m == 0) { o.u = sign; return o.f; }
        float v = (float)m * 5.9604644775390625e-8f; /* m * 2^-24, exact */
        return sign ? -v : v;
    }
    if (e == 31) o.u = sign | 0x7f800000u | (m << 13);
    else o.u = sign | ((e + 112) << 23) | (m << 13);
    return o.f;
}

static float lerpf(float a, float b, float t) { return fmaf(t, b - a, a); }

/* inverse of the GL matrix whose column-major storage is `gl` (16 floats),
 * by cofactor expansion in double; out[r*4+c] = inverse[r][c] as float */
static int invert_gl(const float *gl, float *out) {
    double m[4][4];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) m[r][c] = (double)gl[c * 4 + r];
    double cof[4][4];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            double s[3][3];
            int rr = 0;
            for (int i = 0; i < 4; ++i) {
                if (i == r) continue;
                int cc = 0;
                for (int j = 0; j < 4; ++j) {
                    if (j == c) continue;
                    s[rr][cc++] = m[i][j];
                }
                ++rr;
            }
            double det3 = s[0][0] * (s[1][1] * s[2][2] - s[1][2] * s[2][1])
                        - s[0][1] * (s[1][0] * s[2][2] - s[1][2] * s[2][0])
                        + s[0][2] * (s[1][0] * s[2][1] - s[1][1] * s[2][0]);
            cof[r][c] = ((r + c) & 1) ? -det3 : det3;
        }
    double det = 0.0;
    for (int c = 0; c < 4; ++c) det += m[0][c] * cof[0][c];
    if (det == 0.0 || det != det) return -1;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[r * 4 + c] = (float)(cof[c][r] / det);
    return 0;
}

typedef struct {
    float ip[8], iv[12];
    float light_dir[3];
    float inv_ext[3];
    float alpha_k;
    int ext[3];          /* extent along world x, y, z = W, H, D */
    long long stride[3]; /* element stride along world x, y, z   */
} Derived;

static float fetch(const OracleScene *s, long long idx) {
    switch (s->dtype) {
    case ORACLE_U8: return (float)((const uint8_t *)s->volume)[idx];
    case ORACLE_F16: return half_to_float(((const uint16_t *)s->volume)[idx]);
    default: return ((const float *)s->volume)[idx];
    }
}

/* One ray of volume.frag.glsl:main (lines 70-122). Returns in-box samples. */
static int march_pixel(const OracleScene *s, const Derived *dv, int px, int py, float out[4]) {
    /* vertex stage + ray_direction (vert:8, frag:47-54) */
    float uvx = ((float)px + 0.5f) / (float)s->width;
    float uvy = ((float)py + 0.5f) / (float)s->height;
    float nx = uvx * 2.0f - 1.0f, ny = uvy * 2.0f - 1.0f;
    const float *ip = dv->ip, *iv = dv->iv;
    float ex = ((ip[0] * nx + ip[1] * ny) + ip[2] * -1.0f) + ip[3] * 1.0f;
    float ey = ((ip[4] * nx + ip[5] * ny) + ip[6] * -1.0f) + ip[7] * 1.0f;
    float w[3];
    for (int r = 0; r < 3; ++r)
        w[r] = ((iv[r * 4 + 0] * ex + iv[r * 4 + 1] * ey) + iv[r * 4 + 2] * -1.0f) + iv[r * 4 + 3] * 0.0f;
    float wl = 1.0f / sqrtf((w[0] * w[0] + w[1] * w[1]) + w[2] * w[2]);
    float dir[3] = {w[0] * wl, w[1] * wl, w[2] * wl};
    const float *o = s->cam_pos;

    /* intersect_box (frag:56-68) */
    float tn = -INFINITY, tf = INFINITY;
    for (int a = 0; a < 3; ++a) {
        float inv = 1.0f / dir[a];
        float t0 = (s->bmin[a] - o[a]) * inv, t1 = (s->bmax[a] - o[a]) * inv;
        float lo = fminf(t0, t1), hi = fmaxf(t0, t1);
        tn = a == 0 ? lo : fmaxf(tn, lo);
        tf = a == 0 ? hi : fminf(tf, hi);
    }
    out[0] = out[1] = out[2] = out[3] = 0.0f;
    if (!(tn <= tf && tf > 0.0f)) return 0;            /* frag:75-78 */
    tn = fmaxf(tn, 0.0f);                               /* frag:80 */
    float pos[3], dstep[3];
    for (int a = 0; a < 3; ++a) {
        pos[a] = o[a] + dir[a] * tn;                    /* frag:81 */
        dstep[a] = dir[a] * s->step_size;               /* frag:118 */
    }

    float acc_r = 0.0f, acc_g = 0.0f, acc_b = 0.0f, acc_a = 0.0f;
    int samples = 0;
    for (int i = 0; i < s->max_steps && acc_a < 0.99f; ++i) {     /* frag:87 */
        float t[3];
        int valid = 1;
        for (int a = 0; a < 3; ++a) {                   /* frag:88-92, 25-27, 41-45 */
            t[a] = (pos[a] - s->bmin[a]) * dv->inv_ext[a];
            valid &= (t[a] >= 0.0f) & (t[a] <= 1.0f);
        }
        if (valid) {
            ++samples;
            /* texture(volume_texture, tex.zyx): texel centres, clamp to edge */
            long long i0[3], i1[3];
            float f[3];
            for (int a = 0; a < 3; ++a) {
                float u = t[a] * (float)dv->ext[a] - 0.5f;
                float fl = floorf(u);
                f[a] = u - fl;
                long long k0 = (long long)fl, k1 = k0 + 1;
                if (k0 < 0) k0 = 0;
                if (k1 > dv->ext[a] - 1) k1 = dv->ext[a] - 1;
                i0[a] = k0 * dv->stride[a];
                i1[a] = k1 * dv->stride[a];
            }
            /* lerp along z (texture s), then y (t), then x (r) */
            float v[2][2];
            for (int xi = 0; xi < 2; ++xi)
                for (int yi = 0; yi < 2; ++yi) {
                    long long b = (xi ? i1[0] : i0[0]) + (yi ? i1[1] : i0[1]);
                    v[xi][yi] = lerpf(fetch(s, b + i0[2]), fetch(s, b + i1[2]), f[2]);
                }
            float density = lerpf(lerpf(v[0][0], v[0][1], f[1]), lerpf(v[1][0], v[1][1], f[1]), f[0]);
            density = density * s->value_scale;

            /* LUT lookup (frag:96): x = d*size - 0.5, two-entry lerp, clamp */
            float lu = density * (float)s->lut_size - 0.5f;
            float lfl = floorf(lu);
            float la = lu - lfl;
            long long l0, l1;
            /* clamp-to-edge on the entry indices; a NaN density reads entry 0 */
            float lf1 = lfl + 1.0f;
            if (!(lfl >= 0.0f)) l0 = 0; else if (lfl > (float)(s->lut_size - 1)) l0 = s->lut_size - 1; else l0 = (long long)lfl;
            if (!(lf1 >= 0.0f)) l1 = 0; else if (lf1 > (float)(s->lut_size - 1)) l1 = s->lut_size - 1; else l1 = (long long)lf1;
            const float *L0 = s->lut + 4 * l0, *L1 = s->lut + 4 * l1;
            float cr = lerpf(L0[0], L1[0], la), cg = lerpf(L0[1], L1[1], la);
            float cb = lerpf(L0[2], L1[2], la), alpha_tf = lerpf(L0[3], L1[3], la);

            /* Beer-Lambert correction (frag:101) */
            float alpha = 1.0f - oracle_expf(-(alpha_tf * dv->alpha_k));

            /* normal (frag:103-104); without a normal texture the sampler reads
             * the R32F volume texture, i.e. (density, 0, 0) */
            float n[3];
            if (s->normals) {
                for (int c = 0; c < 3; ++c) {
                    float nv[2][2];
                    for (int xi = 0; xi < 2; ++xi)
                        for (int yi = 0; yi < 2; ++yi) {
                            long long b = (xi ? i1[0] : i0[0]) + (yi ? i1[1] : i0[1]);
                            nv[xi][yi] = lerpf(s->normals[3 * (b + i0[2]) + c],
                                               s->normals[3 * (b + i1[2]) + c], f[2]);
                        }
                    n[c] = lerpf(lerpf(nv[0][0], nv[0][1], f[1]), lerpf(nv[1][0], nv[1][1], f[1]), f[0]);
                }
            } else {
                n[0] = density; n[1] = 0.0f; n[2] = 0.0f;
            }
            float n2 = (n[0] * n[0] + n[1] * n[1]) + n[2] * n[2];
            float di = 0.0f;                            /* frag:107-110 */
            if (n2 > 0.0f) {
                float inv = (float)(1.0 / sqrt((double)n2));
                float d = ((n[0] * inv) * dv->light_dir[0] + (n[1] * inv) * dv->light_dir[1])
                        + (n[2] * inv) * dv->light_dir[2];
                di = fmaxf(d, 0.0f);
            }
            float light = s->ambient + s->diffuse * di;

            /* front-to-back compositing (frag:112-115) */
            float tr = 1.0f - acc_a;
            acc_r = acc_r + tr * ((cr * light) * alpha);
            acc_g = acc_g + tr * ((cg * light) * alpha);
            acc_b = acc_b + tr * ((cb * light) * alpha);
            acc_a = acc_a + tr * alpha;
        }
        for (int a = 0; a < 3; ++a) pos[a] = pos[a] + dstep[a];  /* frag:118 */
    }
    out[0] = acc_r; out[1] = acc_g; out[2] = acc_b; out[3] = acc_a;
    return samples;
}

static float clamp01(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }

/* GL blend onto a cleared RGBA8 target: RGB = c*a, A = a*a, then UNORM8. */
static uint32_t blend_store(const float c[4]) {
    float a = clamp01(c[3]);
    uint32_t r = (uint32_t)rintf((clamp01(c[0]) * a) * 255.0f);
    uint32_t g = (uint32_t)rintf((clamp01(c[1]) * a) * 255.0f);
    uint32_t b = (uint32_t)rintf((clamp01(c[2]) * a) * 255.0f);
    uint32_t al = (uint32_t)rintf((a * a) * 255.0f);
    return r | (g << 8) | (b << 16) | (al << 24);
}

static int derive(const OracleScene *s, Derived *dv) {
    float ip[16], iv[16];
    if (invert_gl(s->proj, ip) || invert_gl(s->view, iv)) return -1;
    memcpy(dv->ip, ip, 8 * sizeof(float));
    memcpy(dv->iv, iv, 12 * sizeof(float));
    float l[3];
    for (int a = 0; a < 3; ++a) l[a] = s->light_target[a] - s->light_pos[a];
    float l2 = (l[0] * l[0] + l[1] * l[1]) + l[2] * l[2];
    float li = l2 > 0.0f ? 1.0f / sqrtf(l2) : 0.0f;
    for (int a = 0; a < 3; ++a) dv->light_dir[a] = l[a] * li;
    for (int a = 0; a < 3; ++a) dv->inv_ext[a] = 1.0f / (s->bmax[a] - s->bmin[a]);
    dv->alpha_k = s->step_size / s->reference_step_size;
    /* world x <-> texture r (slowest, extent W), y <-> t (H), z <-> s (D) */
    dv->ext[0] = s->dims[2]; dv->ext[1] = s->dims[1]; dv->ext[2] = s->dims[0];
    dv->stride[2] = 1;
    dv->stride[1] = s->dims[0];
    dv->stride[0] = (long long)s->dims[0] * s->dims[1];
    return 0;
}

/* Render the full image.  out8: W*H RGBA8 (bottom row first); outf: W*H*4
 * floats of the pre-blend fragment colour (nullable); counts: W*H in-box
 * sample counts (nullable); samples: total in-box samples (nullable).  Rows [row0, row1) only, when row1 > row0 (lets a
 * caller time a bounded sample of the image).  Returns 0 on success. */
int oracle_render_rows(const OracleScene *s, int row0, int row1, uint8_t *out8, float *outf,
                       int *counts, long long *samples, int nthreads) {
    Derived dv;
    if (derive(s, &dv)) return -1;
    if (row1 <= row0) { row0 = 0; row1 = s->height; }
    long long total = 0;
    int W = s->width;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
#endif
    for (int py = row0; py < row1; ++py) {
        for (int px = 0; px < W; ++px) {
            float c[4];
            int n = march_pixel(s, &dv, px, py, c);
            total += n;
            long long idx = (long long)py * W + px;
            if (counts) counts[idx] = n;
            if (out8) {
                uint32_t v = blend_store(c);
                memcpy(out8 + 4 * idx, &v, 4);
            }
            if (outf) memcpy(outf + 4 * idx, c, 16);
        }
    }
    if (samples) *samples = total;
    return 0;
}

int oracle_render(const OracleScene *s, uint8_t *out8, float *outf, long long *samples,
                  int nthreads) {
    return oracle_render_rows(s, 0, 0, out8, outf, NULL, samples, nthreads);
}

/* the derived per-frame constants, in the layout of pvr_frame_constants */
int oracle_frame_constants(const OracleScene *s, float out[27]) {
    Derived dv;
    if (derive(s, &dv)) return -1;
    memcpy(out, dv.ip, 8 * sizeof(float));
    memcpy(out + 8, dv.iv, 12 * sizeof(float));
    memcpy(out + 20, dv.light_dir, 3 * sizeof(float));
    memcpy(out + 23, dv.inv_ext, 3 * sizeof(float));
    out[26] = dv.alpha_k;
    return 0;
}

/* exposed for tests of the exp restatement */
void oracle_expf_array(const float *x, float *y, long long n) {
    for (long long i = 0; i < n; ++i) y[i] = oracle_expf(x[i]);
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
