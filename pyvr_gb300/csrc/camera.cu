// Host-side camera setup of the batch and serving paths, in double precision:
// the orbit camera of pyvr/camera/control.py:238-351 (azimuth about init_up,
// elevation about init_up x view_dir, roll about view_dir, composed
// azimuth*elevation*roll, applied to the distance-scaled initial offset) and
// the matrices of pyvr/camera/camera.py:292-369, produced as the float32
// arrays the reference renderer sends as uniforms (renderer.py:160-172).
// The reference works in float32 up to the rotations; here every step before
// the final float32 rounding is double, so entries agree with the
// reference's to float32 rounding (a few ulp at most).
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

// Rotation of v by |r| radians about r (Rodrigues).
V3 rotate(V3 v, V3 r) {
    const double th = norm(r);
    if (th == 0.0) return v;
    const V3 k = mul(r, 1.0 / th);
    const double c = std::cos(th), s = std::sin(th);
    return add(add(mul(v, c), mul(cross(k, v), s)), mul(k, dot(k, v) * (1.0 - c)));
}

V3 f3(const float *p) { return {p[0], p[1], p[2]}; }

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
    const V3 tgt = f3(target), up0 = f3(init_up);
    V3 off = sub(f3(init_pos), tgt);
    const double n = norm(off);
    if (n == 0.0) return pvr::fail(PVR_ERR_VALUE, "init_pos must not be the zero vector (relative to target)");
    off = mul(off, distance / n);
    const V3 view_dir = mul(off, -1.0 / norm(off));
    V3 ax = cross(up0, view_dir);
    double al = norm(ax);
    if (al < 1e-6) {  // init_up parallel to the view direction
        const V3 alt = std::fabs(up0.x) < 0.9 ? V3{1.0, 0.0, 0.0} : V3{0.0, 0.0, 1.0};
        ax = cross(up0, alt);
        al = norm(ax);
    }
    ax = mul(ax, 1.0 / al);
    // rot = R_az * R_el * R_roll: apply roll first, then elevation, then azimuth
    auto apply = [&](V3 v) {
        return rotate(rotate(rotate(v, mul(view_dir, roll)), mul(ax, elevation)), mul(up0, azimuth));
    };
    const V3 pos = add(apply(off), tgt);
    const V3 up = apply(up0);
    // lookAt, basis in the first three columns of the row-major array
    V3 fwd = sub(tgt, pos);
    fwd = mul(fwd, 1.0 / norm(fwd));
    V3 right = cross(fwd, up);
    const double rl = norm(right);
    // up (nearly) parallel to the view direction: the basis is decided by
    // rounding noise (the reference's own matrices included), so no answer
    // here would reproduce it; the caller takes the matrices from elsewhere
    if (!(rl >= 1e-6))
        return pvr::fail(PVR_ERR_VALUE, "up vector parallel to the view direction: view matrix undefined");
    right = mul(right, 1.0 / rl);
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
