// Per-frame constants, computed on the host once per launch: the camera
// geometry of castRay / reprojection / TXAA (ViewConsts in mt_kernels.h:
// camera basis, slot jitter, ref, the inner shell's origin terms) and the
// raymarch's frame terms (Frame: shell radii and reciprocals, wind and skew,
// the per-step jitter, the sun direction and cone-light kernel of
// ray_consts, the sky's sun terms, the FP64 shell intersections' origin
// terms).  Each value is the result of the same operations, in the same
// order, that the shaders perform per pixel or per ray (cloudRayMarch.comp
// castRay / getJitterOffset :114-226, raySphereIntersection :229-273, the
// cone set-up :598-624, the sky :401-467), so the kernels give the bits they
// gave when each pixel or ray computed them -- the IEEE operations exactly;
// the sky's acos / pow / exp are the host's, within a few ulp of the
// device's.  Built with -ffp-contract=off: no fused multiply-add may change
// a rounding.
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
    // ray_consts' sun direction and cone-light kernel, in its order of operations
    float ld[3];
    normalize(ld, p.sun_light_pos[0] - f->eye[0], p.sun_light_pos[1] - f->eye[1], p.sun_light_pos[2] - f->eye[2]);
    for (int i = 0; i < 3; ++i) f->light_dir[i] = ld[i];
    {
        const float ax = std::fabs(ld[0]), ay = std::fabs(ld[1]), az = std::fabs(ld[2]);
        float mc[3] = {0.0f, 0.0f, 0.0f};
        if (ax > ay && ax > az)
            mc[0] = ax;
        else if (ay > ax && ay > az)
            mc[1] = ay;
        else
            mc[2] = az;
        auto cross = [](float o[3], const float a[3], const float b[3]) {
            o[0] = a[1] * b[2] - b[1] * a[2];
            o[1] = a[2] * b[0] - b[2] * a[0];
            o[2] = a[0] * b[1] - b[0] * a[1];
        };
        float zc[3], xc[3];
        cross(zc, ld, mc);
        cross(xc, zc, ld);
        static const float k[6][3] = {{0.1f, 0.25f, -0.15f}, {0.2f, 0.5f, 0.2f},   {-0.2f, 0.1f, -0.1f},
                                      {-0.05f, 0.75f, 0.05f}, {-0.1f, 1.0f, 0.0f}, {0.0f, 3.0f, 0.0f}};
        for (int i = 0; i < 6; ++i)
            for (int c = 0; c < 3; ++c)  // mat3(xC, lightDir, zC) * k[i]
                f->cone[i][c] = xc[c] * k[i][0] + ld[c] * k[i][1] + zc[c] * k[i][2];
    }
    // atmosphere_color's sun terms, in its order of operations
    {
        float sd[3], ss[3];
        normalize(sd, p.sky_sun_pos[0] - f->eye[0], p.sky_sun_pos[1] - f->eye[1], p.sky_sun_pos[2] - f->eye[2]);
        normalize(ss, p.sky_sun_pos[0], p.sky_sun_pos[1], p.sky_sun_pos[2]);
        auto gmin_ = [](float a, float b) { return b < a ? b : a; };
        auto gmax_ = [](float a, float b) { return a < b ? b : a; };
        const float zc = gmin_(gmax_(ss[1], -1.0f), 1.0f);
        const float sunI =
            1000.0f * gmax_(0.0f, 1.0f - std::pow(2.718281828459f, -((1.6110731557f - std::acos(zc)) / 1.5f)));
        const float sunFade = 1.0f - gmin_(gmax_(1.0f - std::exp(p.sky_sun_pos[1] / 450000.0f), 0.0f), 1.0f);
        static const float RT[3] = {5.804542996261093E-6f, 1.3562911419845635E-5f, 3.0265902468824876E-5f};
        static const float MIE[3] = {1.839991851443397f, 2.779802391966052f, 4.079047954386109f};
        const float rs = 2.0f - 1.0f + sunFade;
        const float c = (0.2f * 10.0f) * 10E-18f;
        for (int i = 0; i < 3; ++i) {
            f->sky_sun_dir[i] = sd[i];
            f->sky_betaR[i] = RT[i] * rs;
            f->sky_betaM[i] = ((0.434f * c) * MIE[i]) * 0.005f;
            f->sky_betaRM[i] = f->sky_betaR[i] + f->sky_betaM[i];
        }
        f->sky_sunE = 0.780f * sunI;
        float yd = 1.0f - sd[1];
        f->sky_yDot = yd * (yd * yd * yd * yd);
    }
    // ray_sphere's and ray_sphere_fp64's origin terms, in their orders of operations
    const float radii[2] = {f->Rin, f->Rout};
    for (int s = 0; s < 2; ++s) {
        for (int i = 0; i < 3; ++i) f->sh32_o[s][i] = (f->eye[i] - f->ec[i]) / radii[s];
        const float* o = f->sh32_o[s];
        f->sh32_c[s] = (o[0] * o[0] + o[1] * o[1] + o[2] * o[2]) - 1.0f;
    }
    for (int s = 0; s < 2; ++s) {
        const double r = (double)radii[s];
        for (int i = 0; i < 3; ++i) f->sh_o[s][i] = ((double)f->eye[i] - (double)f->ec[i]) / r;
        const double* o = f->sh_o[s];
        f->sh_c[s] = (o[0] * o[0] + o[1] * o[1] + o[2] * o[2]) - 1.0;
    }
}

}  // namespace mt
