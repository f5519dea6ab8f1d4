// Per-frame constants of the reprojection / TXAA geometry (ViewConsts in
// mt_kernels.h), computed on the host once per launch.  Every value is the
// IEEE FP32 result of the same operations, in the same order, that the
// per-pixel code performs (cast_ray, jitter_offset and ray_sphere of
// mt_shared.cuh), so the kernels give the same bits as when each pixel
// computed them.  Built with -ffp-contract=off: no fused multiply-add may
// change a rounding.
#include <cmath>
#include <cuda_runtime.h>

#include "mt_kernels.h"

namespace mt {

namespace {

void normalize(float out[3], float x, float y, float z) {
    const float l = std::sqrt(x * x + y * y + z * z);
    out[0] = x / l;
    out[1] = y / l;
    out[2] = z / l;
}

// cloudRayMarch.comp:114-132; reprojection.comp:72-90 reads halton 1/2 again
// for index >= 4 (`repro`).
void jitter(const mt_time_ubo& tm, int index, float dimx, float dimy, bool repro, float& jx, float& jy) {
    index = index / 2;
    float x, y;
    if (index < 4) {
        x = tm.halton_seq1[index];
        y = tm.halton_seq2[index];
    } else {
        index -= 4;
        x = repro ? tm.halton_seq1[index] : tm.halton_seq3[index];
        y = repro ? tm.halton_seq2[index] : tm.halton_seq4[index];
    }
    jx = x / dimx;
    jy = y / dimy;
}

void rcp(float out[2], float b) {
    out[0] = b;
    out[1] = 1.0f / b;
}

}  // namespace

void make_view_consts(ViewConsts* v, const mt_params& p, const mt_camera_ubo& cam, const mt_camera_ubo& cam_old,
                      const mt_time_ubo& tm, int W, int H, bool repro) {
    for (int i = 0; i < 3; ++i) v->eye[i] = p.eye_sign * cam.eye[i];
    const float* m = cam.view;
    normalize(v->right, m[0], m[4], m[8]);
    normalize(v->up, m[1], m[5], m[9]);
    float look[3];
    normalize(look, m[2], m[6], m[10]);
    for (int i = 0; i < 3; ++i) look[i] = -look[i];
    jitter(tm, tm.frame_count_mod16, (float)W, (float)H, repro, v->jx, v->jy);
    v->tanx = cam.tan_fov_by_2[0];
    v->tany = cam.tan_fov_by_2[1];
    for (int i = 0; i < 3; ++i) v->ref[i] = v->eye[i] + look[i];
    v->ec[0] = v->eye[0];
    v->ec[1] = -p.earth_radius;
    v->ec[2] = v->eye[2];
    v->Rin = p.shell_inner_radius;
    for (int i = 0; i < 3; ++i) v->ro[i] = (v->eye[i] - v->ec[i]) / p.shell_inner_radius;
    v->C = (v->ro[0] * v->ro[0] + v->ro[1] * v->ro[1] + v->ro[2] * v->ro[2]) - 1.0f;
    rcp(v->r_w, (float)W);
    rcp(v->r_h, (float)H);
    rcp(v->r_tanx, v->tanx);
    rcp(v->r_tany, v->tany);
    for (int i = 0; i < 16; ++i) v->ov[i] = cam_old.view[i];
}

void make_march_jitter(float out[16][3], const mt_time_ubo& tm) {
    for (int index = 0; index < 16; ++index) {
        float jx, jy;
        jitter(tm, index, 1.0f, 1.0f, false, jx, jy);
        jx = jx / 75.0f;
        jy = jy / 75.0f;
        out[index][0] = jx;
        out[index][1] = (jx + jy) * 1.180f;
        out[index][2] = jy;
    }
}

void make_march_frame(Frame* f, const mt_params& p, const mt_camera_ubo& cam, const mt_time_ubo& tm) {
    f->R = p.earth_radius;
    f->Rin = p.shell_inner_radius;
    f->Rout = p.shell_outer_radius;
    f->thickness = f->Rout - f->Rin;
    f->inner_alt = f->Rin - f->R;
    f->r_thick = Rcp{f->thickness, 1.0f / f->thickness};
    f->r_period = Rcp{p.noise_period, 1.0f / p.noise_period};
    f->r_weather = Rcp{p.weather_scale, 1.0f / p.weather_scale};
    for (int i = 0; i < 3; ++i) {
        f->eye[i] = p.eye_sign * cam.eye[i];
        f->wind_t[i] = (p.wind_dir[i] * p.wind_speed) * tm.time[1];
        f->skew[i] = p.skew_dir[i];
    }
    f->ec[0] = f->eye[0];
    f->ec[1] = -f->R;
    f->ec[2] = f->eye[2];
    // ray_sphere_fp64's origin terms, in its order of operations
    const float radii[2] = {f->Rin, f->Rout};
    for (int s = 0; s < 2; ++s) {
        const double r = (double)radii[s];
        for (int i = 0; i < 3; ++i) f->sh_o[s][i] = ((double)f->eye[i] - (double)f->ec[i]) / r;
        const double* o = f->sh_o[s];
        f->sh_c[s] = (o[0] * o[0] + o[1] * o[1] + o[2] * o[2]) - 1.0;
    }
}

}  // namespace mt
