// Host-side camera setup of the batch and serving paths, in double precision:
// the orbit camera of pyvr/camera/control.py:238-351 (azimuth about init_up,
// elevation about init_up x view_dir, roll about view_dir, composed
// azimuth*elevation*roll, applied to the distance-scaled initial offset) and
// the matrices of pyvr/camera/camera.py:292-369, produced as the float32
// arrays the reference renderer sends as uniforms (renderer.py:160-172).
// The steps the reference takes in float32 (the offset, the view direction,
// the elevation axis and the rotation vectors) are taken in float32 here too,
// the rotations and the lookAt in double, so that the float32 matrices equal
// the Camera methods' (pyvr_gb300/camera.py) bit for bit but for rounding
// differences of the double steps (library sin/cos, summation order), which
// reach the float32 results very rarely.
#include <cmath>
#include <cstring>

#include "pvr_internal.h"

namespace {

struct V3 {
    double x, y, z;
};
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 mul(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double norm(V3 a) { return std::sqrt(dot(a, a)); }

// float32 vectors, each operation rounded to float (numpy float32 arrays)
struct F3 {
    float x, y, z;
};
F3 fsub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
F3 fdiv(F3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
F3 fmul(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
F3 fneg(F3 a) { return {-a.x, -a.y, -a.z}; }
F3 fcross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
// the float32 Euclidean norm: the exact sum of squares rounded once, its
// square root rounded to float
float fnorm(F3 a) {
    const double s = (double)a.x * a.x + (double)a.y * a.y + (double)a.z * a.z;
    return (float)std::sqrt((double)(float)s);
}
V3 wide(F3 a) { return {a.x, a.y, a.z}; }

struct M3 {
    double m[3][3];
};

// Rotation matrix by |r| radians about r: I + sin(t) K + (1 - cos(t)) K^2
// with K the cross-product matrix of r / |r|, evaluated in that order.
M3 axis_angle(V3 r) {
    M3 out = {{{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}};
    const double th = std::sqrt(dot(r, r));
    if (th == 0.0) return out;
    const V3 k = {r.x / th, r.y / th, r.z / th};
    const double K[3][3] = {{0.0, -k.z, k.y}, {k.z, 0.0, -k.x}, {-k.y, k.x, 0.0}};
    double K2[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) K2[i][j] = K[i][0] * K[0][j] + K[i][1] * K[1][j] + K[i][2] * K[2][j];
    const double s = std::sin(th), c1 = 1.0 - std::cos(th);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) out.m[i][j] = out.m[i][j] + s * K[i][j] + c1 * K2[i][j];
    return out;
}

M3 matmul(const M3 &a, const M3 &b) {
    M3 out;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) out.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j];
    return out;
}

V3 apply(const M3 &a, V3 v) {
    return {a.m[0][0] * v.x + a.m[0][1] * v.y + a.m[0][2] * v.z, a.m[1][0] * v.x + a.m[1][1] * v.y + a.m[1][2] * v.z,
            a.m[2][0] * v.x + a.m[2][1] * v.y + a.m[2][2] * v.z};
}

}  // namespace

extern "C" int pvr_camera_spherical(const float target[3], double azimuth, double elevation, double roll,
                                    double distance, const float init_pos[3], const float init_up[3],
                                    double fov, double near_plane, double far_plane, double aspect,
                                    float view_out[16], float proj_out[16], float pos_out[3]) {
    if (!target || !init_pos || !init_up || !view_out || !proj_out || !pos_out)
        return pvr::fail(PVR_ERR_VALUE, "NULL argument");
    if (!(distance > 0.0)) return pvr::fail(PVR_ERR_VALUE, "distance must be positive");
    if (!(fov > 0.0 && fov < M_PI)) return pvr::fail(PVR_ERR_VALUE, "fov must be between 0 and pi radians");
    if (!(near_plane > 0.0) || !(far_plane > near_plane) || !(aspect > 0.0))
        return pvr::fail(PVR_ERR_VALUE, "invalid near/far/aspect");
    // float32 up to the rotations, as the reference computes it
    // (pyvr/camera/control.py:276-314): the offset, the view direction, the
    // elevation axis and the three rotation vectors are float32 arrays
    const F3 tgt = {target[0], target[1], target[2]};
    const F3 up0 = {init_up[0], init_up[1], init_up[2]};
    F3 off = fsub({init_pos[0], init_pos[1], init_pos[2]}, tgt);
    const float n = fnorm(off);
    if (n == 0.0f) return pvr::fail(PVR_ERR_VALUE, "init_pos must not be the zero vector (relative to target)");
    off = fmul(fdiv(off, n), (float)distance);
    const F3 view_dir = fdiv(fneg(off), fnorm(off));
    F3 ax = fcross(up0, view_dir);
    float al = fnorm(ax);
    if (al < 1e-6f) {  // init_up parallel to the view direction
        const F3 alt = std::fabs(up0.x) < 0.9f ? F3{1.0f, 0.0f, 0.0f} : F3{0.0f, 0.0f, 1.0f};
        ax = fcross(up0, alt);
        al = fnorm(ax);
    }
    ax = fdiv(ax, al);
    // rot = R(azimuth about init_up) R(elevation about the elevation axis)
    // R(roll about the view direction), in double from the float32 vectors
    const M3 rot = matmul(matmul(axis_angle(wide(fmul(up0, (float)azimuth))),
                                 axis_angle(wide(fmul(ax, (float)elevation)))),
                          axis_angle(wide(fmul(view_dir, (float)roll))));
    const V3 pos = add(apply(rot, wide(off)), wide(tgt));
    const V3 up = apply(rot, wide(up0));
    // lookAt, basis in the first three columns of the row-major array
    // (pyvr/camera/camera.py:292-334)
    V3 fwd = sub(wide(tgt), pos);
    fwd = mul(fwd, 1.0 / norm(fwd));
    V3 right = cross(fwd, up);
    const double rl = norm(right);
    // up (nearly) parallel to the view direction: the basis is decided by
    // rounding noise (the reference's own matrices included), so no answer
    // here would reproduce it; the caller takes the matrices from elsewhere
    if (!(rl >= 1e-6))
        return pvr::fail(PVR_ERR_VALUE, "up vector parallel to the view direction: view matrix undefined");
    right = {right.x / rl, right.y / rl, right.z / rl};
    const V3 upc = cross(right, fwd);
    const double m[16] = {right.x, upc.x, -fwd.x, 0.0, right.y, upc.y, -fwd.y, 0.0,
                          right.z, upc.z, -fwd.z, 0.0, -dot(right, pos), -dot(upc, pos), dot(fwd, pos), 1.0};
    for (int i = 0; i < 16; ++i) view_out[i] = (float)m[i];
    const double f = 1.0 / std::tan(fov / 2.0);
    const double p[16] = {f / aspect, 0.0, 0.0, 0.0, 0.0, f, 0.0, 0.0,
                          0.0, 0.0, (far_plane + near_plane) / (near_plane - far_plane),
                          (2.0 * far_plane * near_plane) / (near_plane - far_plane), 0.0, 0.0, -1.0, 0.0};
    for (int i = 0; i < 16; ++i) proj_out[i] = (float)p[i];
    pos_out[0] = (float)pos.x;
    pos_out[1] = (float)pos.y;
    pos_out[2] = (float)pos.z;
    return PVR_OK;
}
