// Differentiable march: gradients of an image loss with respect to the RGBA
// LUT and the voxel values (FP32 volume), for several views of one scene.
//
// Forward: the march of pyvr/shaders/volume.frag.glsl:70-122 with the
// renderer's exact per-sample arithmetic (setup_ray, texel fractions,
// z-then-y-then-x trilinear lerps, LUT lerp, pvr_expf opacity correction,
// Lambert term, front-to-back compositing), reading the volume in its linear
// (D, H, W) layout, so the float image equals the renderer's float image.
// Per pixel it also keeps the number of loop iterations executed; nothing
// is kept per sample.
//
// Backward: a second march over each ray in reverse order.  With T_i the
// transmittance in front of sample i, c_i = light_i * rgb_i and
// R_i the radiance behind sample i as seen from just after it,
//   C = sum_i T_i alpha_i c_i,   A = 1 - prod_i (1 - alpha_i),
//   dC/dc_i = T_i alpha_i,       dC/dalpha_i = T_i (c_i - R_i),
//   dA/dalpha_i = T_i (1 - Ra_i),   Ra_i = 1 - prod_{j>i} (1 - alpha_j),
// and walking from the last sample to the first, T_i = T_{i+1} / (1 - alpha_i)
// starting from T_N = 1 - A, R_{i-1} = alpha_i c_i + (1 - alpha_i) R_i,
// Ra_{i-1} = alpha_i + (1 - alpha_i) Ra_i.  The sample positions are those of
// the forward march bit for bit: the position recurrence (repeated float
// additions of one step) is replayed from the ray's start in segments of
// kSeg iterations, each segment buffered and then walked backwards.  A
// sample with alpha exactly 1 (transmittance not recoverable by division)
// takes its T from a forward replay instead.
//
// Chain rule down to the leaves: alpha = 1 - exp(-a K) gives
// dalpha/da = K exp(-a K); the LUT lerp rgba = lerp(lut[i0], lut[i1], f)
// gives weights (1 - f, f) to the two entries and d rgba/d density =
// (lut[i1] - lut[i0]) * lut_size; density = value_scale * trilinear(voxels)
// gives each of the 8 corners its trilinear weight.  Normals (given, or
// (density, 0, 0) without a normal volume) are held constant.  LUT gradients
// are summed per warp over the lanes that address the same entries, then in
// shared memory per block, and added to global memory once per block; voxel
// gradients are added with global atomics.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "pvr_device.cuh"
#include "pvr_internal.h"

namespace pvr {
namespace {

constexpr int kDiffMaxViews = 32;   // views per launch (more are split)
constexpr int kDiffThreads = 256;   // 16 x 16 pixel tile; warps cover 8 x 4 pixels
constexpr int kDiffTile = 16;
constexpr int kSeg = 16;            // reverse-march segment (iterations), buffered in shared memory
constexpr int kDiffMaxLut = 2048;   // LUT entries (shared-memory gradient)

struct DiffParams {
    const float *vol;       // (D, H, W) C order: texel (x, y, z) at (x * H + y) * D + z
    const float *nrm;       // 3 floats per texel, or null
    const float4 *lut;
    float4 *image;          // [view][y][x]
    int *steps;             // [view][y][x] loop iterations executed
    const float4 *gimage;   // dL/dimage
    float4 *glut;           // dL/dlut, accumulated; or null
    float *gvol;            // dL/dvoxel, accumulated; or null
    int nviews, tiles_x, tiles_y;
    int ext[3];             // texels along world x, y, z (W, H, D)
    MarchFrame f[kDiffMaxViews];
};

struct Sample {
    int x0, x1, y0, y1, z0, z1;
    float fx, fy, fz;
    float density;
    int i0, i1;
    float la;
    float4 A, B;
    float r, g, b;   // LUT colour
    float e;         // exp(-a K)
    float alpha;     // 1 - e
    float light;     // ambient + diffuse * max(dot(n, L), 0)
};

__device__ __forceinline__ int texel(const DiffParams &p, int x, int y, int z) {
    return (x * p.ext[1] + y) * p.ext[2] + z;
}

__device__ __forceinline__ int lut_idx(float fl, float lmax, int size) {
    return !(fl >= 0.0f) ? 0 : (fl > lmax ? size - 1 : (int)fl);
}

// texture coordinate of a world position (frag:25-27, 88) and its validity
__device__ __forceinline__ bool tex_coords(const MarchFrame &f, const float pos[3], float t[3]) {
#pragma unroll
    for (int a = 0; a < 3; ++a) t[a] = __fmul_rn(__fadd_rn(pos[a], -f.bmin[a]), f.inv_ext[a]);
    return t[0] >= 0.0f && t[0] <= 1.0f && t[1] >= 0.0f && t[1] <= 1.0f && t[2] >= 0.0f && t[2] <= 1.0f;
}

// once the ray has left the valid run, or cannot reach it, the march ends
__device__ __forceinline__ bool never_valid(const float t[3], const float d[3]) {
    bool nv = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) nv = nv || (t[a] < 0.0f && d[a] <= 0.0f) || (t[a] > 1.0f && d[a] >= 0.0f);
    return nv;
}

__device__ __forceinline__ float tri(const float *v, const DiffParams &p, const Sample &s, int stride, int c) {
    const float v000 = __ldg(v + texel(p, s.x0, s.y0, s.z0) * stride + c);
    const float v001 = __ldg(v + texel(p, s.x0, s.y0, s.z1) * stride + c);
    const float v010 = __ldg(v + texel(p, s.x0, s.y1, s.z0) * stride + c);
    const float v011 = __ldg(v + texel(p, s.x0, s.y1, s.z1) * stride + c);
    const float v100 = __ldg(v + texel(p, s.x1, s.y0, s.z0) * stride + c);
    const float v101 = __ldg(v + texel(p, s.x1, s.y0, s.z1) * stride + c);
    const float v110 = __ldg(v + texel(p, s.x1, s.y1, s.z0) * stride + c);
    const float v111 = __ldg(v + texel(p, s.x1, s.y1, s.z1) * stride + c);
    const float c0 = lerp_tex(lerp_tex(v000, v001, s.fz), lerp_tex(v010, v011, s.fz), s.fy);
    const float c1 = lerp_tex(lerp_tex(v100, v101, s.fz), lerp_tex(v110, v111, s.fz), s.fy);
    return lerp_tex(c0, c1, s.fx);
}

// Everything one in-box sample computes (frag:93-110), with the renderer's
// rounding.  full: also the colour and the light term.
__device__ __forceinline__ void eval_sample(const DiffParams &p, const MarchFrame &f, const float t[3],
                                           bool full, Sample &s) {
    int lo[3], hi[3];
    float fr[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float u = __fadd_rn(__fmul_rn(t[a], f.fext[a]), -0.5f);
        const float fl = floorf(u);
        fr[a] = __fadd_rn(u, -fl);
        const int k = (int)fl;  // -1 .. ext-1
        lo[a] = max(k, 0);
        hi[a] = min(k + 1, p.ext[a] - 1);
    }
    s.x0 = lo[0]; s.x1 = hi[0]; s.y0 = lo[1]; s.y1 = hi[1]; s.z0 = lo[2]; s.z1 = hi[2];
    s.fx = fr[0]; s.fy = fr[1]; s.fz = fr[2];
    s.density = __fmul_rn(tri(p.vol, p, s, 1, 0), f.value_scale);
    // texture(transfer_function_lut, vec2(density, 0.5)) (frag:96)
    const float lu = __fadd_rn(__fmul_rn(s.density, f.flut_size), -0.5f);
    const float lfl = floorf(lu);
    s.la = __fadd_rn(lu, -lfl);
    const float lmax = (float)(f.lut_size - 1);
    s.i0 = lut_idx(lfl, lmax, f.lut_size);
    s.i1 = lut_idx(__fadd_rn(lfl, 1.0f), lmax, f.lut_size);
    s.A = __ldg(p.lut + s.i0);
    s.B = __ldg(p.lut + s.i1);
    const float a_tf = lerp_tex(s.A.w, s.B.w, s.la);
    s.e = pvr_expf(-__fmul_rn(a_tf, f.alpha_k));
    s.alpha = __fadd_rn(1.0f, -s.e);
    if (!full) return;
    s.r = lerp_tex(s.A.x, s.B.x, s.la);
    s.g = lerp_tex(s.A.y, s.B.y, s.la);
    s.b = lerp_tex(s.A.z, s.B.z, s.la);
    float n[3];
    if (p.nrm) {
        n[0] = tri(p.nrm, p, s, 3, 0);
        n[1] = tri(p.nrm, p, s, 3, 1);
        n[2] = tri(p.nrm, p, s, 3, 2);
    } else {  // the reference's unbound normal sampler reads the volume
        n[0] = s.density;
        n[1] = 0.0f;
        n[2] = 0.0f;
    }
    const float n2 = __fadd_rn(__fadd_rn(__fmul_rn(n[0], n[0]), __fmul_rn(n[1], n[1])), __fmul_rn(n[2], n[2]));
    float di = 0.0f;
    if (n2 > 0.0f) {
        const float inv = __frsqrt_rn(n2);  // as the renderer: rsqrt rounded once
        const float d = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(n[0], inv), f.light_dir[0]),
                                            __fmul_rn(__fmul_rn(n[1], inv), f.light_dir[1])),
                                  __fmul_rn(__fmul_rn(n[2], inv), f.light_dir[2]));
        di = fmaxf(d, 0.0f);
    }
    s.light = __fadd_rn(f.ambient, __fmul_rn(f.diffuse, di));
}

__device__ __forceinline__ void pixel_of(int tile_in_view, int tiles_x, int &px, int &py) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    px = (tile_in_view % tiles_x) * kDiffTile + (warp & 1) * 8 + (lane & 7);
    py = (tile_in_view / tiles_x) * kDiffTile + (warp >> 1) * 4 + (lane >> 3);
}

__global__ void __launch_bounds__(kDiffThreads)
diff_forward_kernel(const __grid_constant__ DiffParams p) {
    const int per_view = p.tiles_x * p.tiles_y;
    const int view = blockIdx.x / per_view;
    const MarchFrame &f = p.f[view];
    int px, py;
    pixel_of(blockIdx.x % per_view, p.tiles_x, px, py);
    if (px >= f.width || py >= f.height) return;
    float acc_r = 0.0f, acc_g = 0.0f, acc_b = 0.0f, acc_a = 0.0f;
    int i = 0;
    float pos[3], d[3];
    if (setup_ray(f, px, py, pos, d)) {
        bool entered = false;
        for (;; ++i) {
            if (!(i < f.max_steps && acc_a < 0.99f)) break;
            float t[3];
            if (tex_coords(f, pos, t)) {
                entered = true;
                Sample s;
                eval_sample(p, f, t, true, s);
                // acc.c += (1 - acc.a) * (c * light * alpha); acc.a += (1 - acc.a) * alpha
                const float tr = __fadd_rn(1.0f, -acc_a);
                acc_r = __fadd_rn(acc_r, __fmul_rn(tr, __fmul_rn(__fmul_rn(s.r, s.light), s.alpha)));
                acc_g = __fadd_rn(acc_g, __fmul_rn(tr, __fmul_rn(__fmul_rn(s.g, s.light), s.alpha)));
                acc_b = __fadd_rn(acc_b, __fmul_rn(tr, __fmul_rn(__fmul_rn(s.b, s.light), s.alpha)));
                acc_a = __fadd_rn(acc_a, __fmul_rn(tr, s.alpha));
            } else if (entered || never_valid(t, d)) {
                break;
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) pos[a] = __fadd_rn(pos[a], d[a]);
        }
    }
    const long long idx = ((long long)view * f.height + py) * f.width + px;
    p.image[idx] = make_float4(acc_r, acc_g, acc_b, acc_a);
    p.steps[idx] = i;
}

// 1 - acc.a just before iteration `upto` of the forward march
__device__ float replay_transmittance(const DiffParams &p, const MarchFrame &f, const float pos0[3],
                                      const float d[3], int upto) {
    float pos[3] = {pos0[0], pos0[1], pos0[2]};
    float acc_a = 0.0f;
    for (int i = 0; i < upto; ++i) {
        float t[3];
        if (tex_coords(f, pos, t)) {
            Sample s;
            eval_sample(p, f, t, false, s);
            acc_a = __fadd_rn(acc_a, __fmul_rn(__fadd_rn(1.0f, -acc_a), s.alpha));
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) pos[a] = __fadd_rn(pos[a], d[a]);
    }
    return __fadd_rn(1.0f, -acc_a);
}

__device__ __forceinline__ void add_voxel_grad(const DiffParams &p, const Sample &s, float gd) {
    const float wx[2] = {1.0f - s.fx, s.fx}, wy[2] = {1.0f - s.fy, s.fy}, wz[2] = {1.0f - s.fz, s.fz};
    const int xs[2] = {s.x0, s.x1}, ys[2] = {s.y0, s.y1}, zs[2] = {s.z0, s.z1};
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            const float wab = gd * wx[a] * wy[b];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const float w = wab * wz[c];
                if (w != 0.0f) atomicAdd(p.gvol + texel(p, xs[a], ys[b], zs[c]), w);
            }
        }
}

// Sums v[0..7] over each group of lanes in `peers` (the lanes of `active`
// with the same key, from __match_any_sync) by a tree over the group's
// ranks; returns true on the group's lowest lane, which then holds the sums.
// Every lane of `active` must call it.
__device__ __forceinline__ bool reduce_peers(unsigned active, unsigned peers, float v[8]) {
    const int lane = threadIdx.x & 31;
    int rank = __popc(peers & ((1u << lane) - 1u));
    unsigned above = lane == 31 ? 0u : peers & (0xffffffffu << (lane + 1));
    bool member = true;  // still holds a partial sum of its group
    while (__any_sync(active, member && above != 0u)) {
        const int next = (member && above) ? __ffs(above) - 1 : lane;
        const bool take = member && above != 0u && !(rank & 1);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const float t = __shfl_sync(active, v[c], next);
            if (take) v[c] += t;
        }
        // the odd ranks have handed their sums down and leave
        const unsigned leaving = __ballot_sync(active, member && (rank & 1));
        if (member && (rank & 1)) member = false;
        above &= ~leaving;
        rank >>= 1;
    }
    return member;
}

__device__ void backward_ray(const DiffParams &p, const MarchFrame &f, int px, int py, long long idx,
                             float *s_glut, float *s_seg) {
    const int nsteps = p.steps[idx];
    if (nsteps <= 0) return;
    const float4 g = p.gimage[idx];
    if (g.x == 0.0f && g.y == 0.0f && g.z == 0.0f && g.w == 0.0f) return;
    float pos0[3], d[3];
    if (!setup_ray(f, px, py, pos0, d)) return;
    const float4 out = p.image[idx];
    float T = __fadd_rn(1.0f, -out.w);
    float Rr = 0.0f, Rg = 0.0f, Rb = 0.0f, Ra = 0.0f;
    // this thread's kSeg x 3 positions, strided by the block size (no bank
    // conflicts between the lanes of a warp)
    float *seg = s_seg + threadIdx.x;
    int end = nsteps;
    while (end > 0) {
        const int start = max(0, end - kSeg);
        float q[3] = {pos0[0], pos0[1], pos0[2]};
        for (int k = 0; k < start; ++k)
#pragma unroll
            for (int a = 0; a < 3; ++a) q[a] = __fadd_rn(q[a], d[a]);
        for (int k = start; k < end; ++k) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                seg[((k - start) * 3 + a) * kDiffThreads] = q[a];
                q[a] = __fadd_rn(q[a], d[a]);
            }
        }
        for (int k = end - 1; k >= start; --k) {
            float t[3];
            const float bpos[3] = {seg[((k - start) * 3 + 0) * kDiffThreads], seg[((k - start) * 3 + 1) * kDiffThreads],
                                   seg[((k - start) * 3 + 2) * kDiffThreads]};
            if (!tex_coords(f, bpos, t)) continue;
            Sample s;
            eval_sample(p, f, t, true, s);
            const float om = 1.0f - s.alpha;
            const float Ti = om > 0.0f ? T / om : replay_transmittance(p, f, pos0, d, k);
            const float cr = s.light * s.r, cg = s.light * s.g, cb = s.light * s.b;
            const float dalpha = Ti * (g.x * (cr - Rr) + g.y * (cg - Rg) + g.z * (cb - Rb) + g.w * (1.0f - Ra));
            const float kc = Ti * s.light * s.alpha;
            const float dr = g.x * kc, dg = g.y * kc, db = g.z * kc;
            const float da = dalpha * f.alpha_k * s.e;
            if (s_glut) {
                // neighbouring rays of a warp mostly address the same LUT
                // entries: the lanes with the same pair of entries sum their
                // contributions first, and one lane per pair adds them
                const float w1 = s.la, w0 = 1.0f - s.la;
                float v[8] = {w0 * dr, w0 * dg, w0 * db, w0 * da, w1 * dr, w1 * dg, w1 * db, w1 * da};
                const unsigned active = __activemask();
                const unsigned peers = __match_any_sync(active, ((unsigned)s.i0 << 16) | (unsigned)s.i1);
                if (reduce_peers(active, peers, v)) {
                    const int n = f.lut_size;  // channel-major: s_glut[c * n + entry]
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        if (v[c] != 0.0f) atomicAdd(s_glut + c * n + s.i0, v[c]);
                        if (v[4 + c] != 0.0f) atomicAdd(s_glut + c * n + s.i1, v[4 + c]);
                    }
                }
            }
            if (p.gvol) {
                const float gd = (dr * (s.B.x - s.A.x) + dg * (s.B.y - s.A.y) + db * (s.B.z - s.A.z) +
                                  da * (s.B.w - s.A.w)) * f.flut_size * f.value_scale;
                if (gd != 0.0f) add_voxel_grad(p, s, gd);
            }
            Rr = cr * s.alpha + om * Rr;
            Rg = cg * s.alpha + om * Rg;
            Rb = cb * s.alpha + om * Rb;
            Ra = s.alpha + om * Ra;
            T = Ti;
        }
        end = start;
    }
}

// Dynamic shared memory: the reverse march's position segments (kSeg x 3
// floats per thread), then the block's LUT gradient (4 x lut_size floats,
// channel-major) when the LUT gradient is wanted.
__global__ void __launch_bounds__(kDiffThreads)
diff_backward_kernel(const __grid_constant__ DiffParams p) {
    extern __shared__ float s_dyn[];
    float *s_seg = s_dyn;
    float *s_glut = s_dyn + kSeg * 3 * kDiffThreads;
    const int lut_floats = 4 * p.f[0].lut_size;
    if (p.glut) {
        for (int k = threadIdx.x; k < lut_floats; k += kDiffThreads) s_glut[k] = 0.0f;
        __syncthreads();
    }
    const int per_view = p.tiles_x * p.tiles_y;
    const int total = per_view * p.nviews;
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int view = tile / per_view;
        const MarchFrame &f = p.f[view];
        int px, py;
        pixel_of(tile % per_view, p.tiles_x, px, py);
        if (px < f.width && py < f.height)
            backward_ray(p, f, px, py, ((long long)view * f.height + py) * f.width + px,
                         p.glut ? s_glut : nullptr, s_seg);
    }
    if (p.glut) {
        __syncthreads();
        float *g = reinterpret_cast<float *>(p.glut);  // (lut_size, 4), entry-major
        const int n = p.f[0].lut_size;
        for (int k = threadIdx.x; k < lut_floats; k += kDiffThreads)
            if (s_glut[k] != 0.0f) atomicAdd(g + 4 * (k % n) + k / n, s_glut[k]);
    }
}

int build_params(const pvr_diff_scene *s, int v0, int nv, DiffParams &p) {
    std::memset(&p, 0, sizeof(p));
    p.vol = s->volume;
    p.nrm = s->normals;
    p.lut = reinterpret_cast<const float4 *>(s->lut);
    p.nviews = nv;
    p.tiles_x = (s->width + kDiffTile - 1) / kDiffTile;
    p.tiles_y = (s->height + kDiffTile - 1) / kDiffTile;
    p.ext[0] = s->w;
    p.ext[1] = s->h;
    p.ext[2] = s->d;
    float light_dir[3];
    light_direction(s->light_pos, s->light_target, light_dir);
    for (int k = 0; k < nv; ++k) {
        const pvr_diff_view &v = s->views[v0 + k];
        MarchFrame &f = p.f[k];
        double ip[16], iv[16];
        if (!invert_gl(v.proj, ip)) return fail(PVR_ERR_VALUE, "view %d: projection matrix is singular", v0 + k);
        if (!invert_gl(v.view, iv)) return fail(PVR_ERR_VALUE, "view %d: view matrix is singular", v0 + k);
        for (int i = 0; i < 8; ++i) f.ip[i] = (float)ip[i];
        for (int i = 0; i < 12; ++i) f.iv[i] = (float)iv[i];
        f.width = s->width;
        f.height = s->height;
        for (int a = 0; a < 3; ++a) {
            f.cam[a] = v.camera_pos[a];
            f.bmin[a] = s->min_bounds[a];
            f.bmax[a] = s->max_bounds[a];
            f.inv_ext[a] = 1.0f / (s->max_bounds[a] - s->min_bounds[a]);
            f.ext[a] = p.ext[a];
            f.fext[a] = (float)p.ext[a];
            f.nb[a] = 0;
            f.light_dir[a] = light_dir[a];
        }
        f.step = s->step_size;
        f.alpha_k = s->step_size / s->reference_step_size;
        f.max_steps = s->max_steps;
        f.ambient = s->ambient;
        f.diffuse = s->diffuse;
        f.value_scale = s->value_scale;
        f.lut_size = s->lut_size;
        f.flut_size = (float)s->lut_size;
    }
    return PVR_OK;
}

int check_scene(const pvr_diff_scene *s) {
    if (!s) return fail(PVR_ERR_VALUE, "scene is NULL");
    if (!s->volume || !s->lut || !s->views) return fail(PVR_ERR_VALUE, "scene without volume, LUT or views");
    if (s->d < 1 || s->h < 1 || s->w < 1 || (long long)s->d * s->h * s->w > (1LL << 31) / 4)
        return fail(PVR_ERR_VALUE, "volume dims must be positive and under 2^29 voxels");
    if (s->lut_size < 1 || s->lut_size > kDiffMaxLut)
        return fail(PVR_ERR_VALUE, "LUT size must be in 1..%d, got %d", kDiffMaxLut, s->lut_size);
    if (s->width < 1 || s->height < 1 || s->width > 16384 || s->height > 16384)
        return fail(PVR_ERR_VALUE, "image size must be in 1..16384");
    if (s->n_views < 1 || s->n_views > 4096) return fail(PVR_ERR_VALUE, "n_views must be in 1..4096");
    if (!(s->step_size > 0.0f) || !std::isfinite(s->step_size) || !(s->reference_step_size > 0.0f) ||
        !std::isfinite(s->reference_step_size) || s->max_steps < 1)
        return fail(PVR_ERR_VALUE, "invalid step_size / reference_step_size / max_steps");
    for (int a = 0; a < 3; ++a)
        if (!(s->max_bounds[a] > s->min_bounds[a])) return fail(PVR_ERR_VALUE, "max_bounds must exceed min_bounds");
    return PVR_OK;
}

}  // namespace
}  // namespace pvr

using pvr::fail;

extern "C" int pvr_diff_forward(const pvr_diff_scene *s, float *d_image, int *d_steps, void *stream) {
    if (int rc = pvr::check_scene(s)) return rc;
    if (!d_image || !d_steps) return fail(PVR_ERR_VALUE, "image / steps buffer is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    const long long frame = (long long)s->width * s->height;
    for (int v0 = 0; v0 < s->n_views; v0 += pvr::kDiffMaxViews) {
        const int nv = std::min(pvr::kDiffMaxViews, s->n_views - v0);
        pvr::DiffParams p;
        if (int rc = pvr::build_params(s, v0, nv, p)) return rc;
        p.image = reinterpret_cast<float4 *>(d_image) + v0 * frame;
        p.steps = d_steps + v0 * frame;
        const int blocks = p.tiles_x * p.tiles_y * nv;
        void *args[] = {&p};
        PVR_CUDA(cudaLaunchKernel((const void *)pvr::diff_forward_kernel, dim3(blocks), dim3(pvr::kDiffThreads),
                                  args, 0, st));
    }
    return PVR_OK;
}

extern "C" int pvr_diff_backward(const pvr_diff_scene *s, const float *d_image, const int *d_steps,
                                 const float *d_grad_image, float *d_grad_lut, float *d_grad_volume,
                                 void *stream) {
    if (int rc = pvr::check_scene(s)) return rc;
    if (!d_image || !d_steps || !d_grad_image) return fail(PVR_ERR_VALUE, "image / steps / gradient buffer is NULL");
    if (!d_grad_lut && !d_grad_volume) return PVR_OK;
    cudaStream_t st = (cudaStream_t)stream;
    int device = 0, sms = 0;
    PVR_CUDA(cudaGetDevice(&device));
    PVR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const size_t smem = (size_t)pvr::kSeg * 3 * pvr::kDiffThreads * sizeof(float) +
                        (d_grad_lut ? (size_t)s->lut_size * 4 * sizeof(float) : 0);
    // more than 48 KB of dynamic shared memory (set on the current device)
    PVR_CUDA(cudaFuncSetAttribute((const void *)pvr::diff_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(pvr::kSeg * 3 * pvr::kDiffThreads * sizeof(float) +
                                        pvr::kDiffMaxLut * 4 * sizeof(float))));
    int per_sm = 0;
    PVR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pvr::diff_backward_kernel, pvr::kDiffThreads,
                                                           smem));
    per_sm = std::max(1, per_sm);
    const long long frame = (long long)s->width * s->height;
    for (int v0 = 0; v0 < s->n_views; v0 += pvr::kDiffMaxViews) {
        const int nv = std::min(pvr::kDiffMaxViews, s->n_views - v0);
        pvr::DiffParams p;
        if (int rc = pvr::build_params(s, v0, nv, p)) return rc;
        p.image = const_cast<float4 *>(reinterpret_cast<const float4 *>(d_image)) + v0 * frame;
        p.steps = const_cast<int *>(d_steps) + v0 * frame;
        p.gimage = reinterpret_cast<const float4 *>(d_grad_image) + v0 * frame;
        p.glut = reinterpret_cast<float4 *>(d_grad_lut);
        p.gvol = d_grad_volume;
        const int tiles = p.tiles_x * p.tiles_y * nv;
        const int blocks = std::min(tiles, sms * per_sm);
        void *args[] = {&p};
        PVR_CUDA(cudaLaunchKernel((const void *)pvr::diff_backward_kernel, dim3(blocks), dim3(pvr::kDiffThreads),
                                  args, smem, st));
    }
    return PVR_OK;
}
