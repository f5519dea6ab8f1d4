// TEST INFRASTRUCTURE — CPU restatement of the reference's uniform producers
// and of the two parameter presets.  Only tests/ and bench.py's CPU legs (the
// reference arm and the CPU baseline) call it, so that those legs build their
// inputs without the product library; tests pin it bit for bit against the
// product's producers.
//
//   orc_halton            Scene::HaltonSequenceAt (Scene.cpp:125-138)
//   orc_time_init         Scene::InitializeTime (Scene.cpp:86-119): Halton(3)
//                         at 1..16, frame 0, time (0, 0)
//   orc_camera_look_at    Camera::RecomputeAttributes + UpdateBuffer
//                         (camera.cpp:31-42, 56-76) with glm 0.9.9's lookAtRH,
//                         perspectiveRH_ZO (camera.h defines
//                         GLM_FORCE_DEPTH_ZERO_TO_ONE), normalize = v *
//                         inversesqrt(dot(v, v)), inversesqrt(x) = 1 / sqrt(x)
//   orc_params_reference  the #defines / literals of cloudRayMarch.comp
//                         (:75-95, :489-497, :515-537, :572, :680, :697-698) and
//                         postProcess_TXAA.frag (:258-266)
//   orc_params_config     the benchmark configurations' parameterisation
//
// Built with -ffp-contract=off like the rest of the oracle.
#include <cmath>
#include <cstring>

#include "../include/meteoros.h"

namespace {

struct V3 {
    float x, y, z;
};

V3 vsub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
float vdot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
V3 vcross(V3 a, V3 b) { return V3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
V3 vscale(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
// glm::normalize: v * inversesqrt(dot(v, v)), inversesqrt(x) = 1 / sqrt(x)
V3 vnormalize(V3 a) { return vscale(a, 1.0f / std::sqrt(vdot(a, a))); }

}  // namespace

extern "C" {

float orc_halton(int index, int base) {
    float f = 1.0f, r = 0.0f;
    for (; index > 0; index /= base) {
        f = f / (float)base;
        r = r + f * (float)(index % base);
    }
    return r;
}

void orc_time_init(mt_time_ubo* t) {
    std::memset(t, 0, sizeof(*t));
    float* rows[4] = {t->halton_seq1, t->halton_seq2, t->halton_seq3, t->halton_seq4};
    for (int i = 1; i <= 16; ++i) rows[(i - 1) / 4][(i - 1) % 4] = orc_halton(i, 3);
}

void orc_camera_look_at(mt_camera_ubo* cam, const float* eye3, const float* ref3, float fovy_deg, float aspect,
                        float znear, float zfar) {
    std::memset(cam, 0, sizeof(*cam));
    const V3 eye{eye3[0], eye3[1], eye3[2]}, ref{ref3[0], ref3[1], ref3[2]};
    // RecomputeAttributes: forward, right, up from the world up (0, 1, 0)
    const V3 fwd = vnormalize(vsub(ref, eye));
    const V3 right = vnormalize(vcross(fwd, V3{0.0f, 1.0f, 0.0f}));
    const V3 up = vcross(right, fwd);
    // lookAtRH(eye, ref, up): columns hold s, u, -f; translation in column 3
    const V3 f = vnormalize(vsub(ref, eye));
    const V3 s = vnormalize(vcross(f, up));
    const V3 u = vcross(s, f);
    float(*V)[4] = reinterpret_cast<float(*)[4]>(cam->view);  // V[column][row]
    V[0][0] = s.x, V[1][0] = s.y, V[2][0] = s.z;
    V[0][1] = u.x, V[1][1] = u.y, V[2][1] = u.z;
    V[0][2] = -f.x, V[1][2] = -f.y, V[2][2] = -f.z;
    V[3][0] = -vdot(s, eye), V[3][1] = -vdot(u, eye), V[3][2] = vdot(f, eye);
    V[3][3] = 1.0f;
    // perspectiveRH_ZO(radians(fovy), aspect, near, far), then proj[1][1] *= -1
    const float rad = fovy_deg * 0.01745329251994329576923690768489f;
    const float th = std::tan(rad / 2.0f);
    float(*P)[4] = reinterpret_cast<float(*)[4]>(cam->proj);
    P[0][0] = 1.0f / (aspect * th);
    P[1][1] = -(1.0f / th);
    P[2][2] = zfar / (znear - zfar);
    P[2][3] = -1.0f;
    P[3][2] = -(zfar * znear) / (zfar - znear);
    cam->eye[0] = eye.x, cam->eye[1] = eye.y, cam->eye[2] = eye.z, cam->eye[3] = 1.0f;
    // tanFovBy2.y = |tan(fovy * 0.5 * (PI / 180.0))| in double, PI = 3.14159 (camera.h)
    cam->tan_fov_by_2[1] = (float)std::fabs(std::tan((double)fovy_deg * 0.5 * (3.14159 / 180.0)));
    cam->tan_fov_by_2[0] = aspect * cam->tan_fov_by_2[1];
}

void orc_params_reference(mt_params* p) {
    std::memset(p, 0, sizeof(*p));
    const float R = 6371000.0f;  // cloudRayMarch.comp:75
    p->earth_radius = R;
    p->shell_inner_radius = R + 7500.0f;
    p->shell_outer_radius = R + 20000.0f;
    p->noise_period = 8.0f;
    p->steps_min = 35, p->steps_max = 60;  // floor(mix(35, 60, 1 - dir.y))
    p->accum_limit = 1.0f;                 // accumDensity >= 1
    p->coverage_mode = 0, p->coverage = 0.6f;
    p->height_gradient = 0;
    p->weather_scale = 60000.0f;
    // wind (1,0,0) + bias (0,0.1,0), times 0.08 * time.y; skew along +x
    p->wind_dir[0] = 1.0f, p->wind_dir[1] = 0.1f, p->wind_dir[2] = 0.0f;
    p->wind_speed = 0.08f;
    p->skew_dir[0] = 1.0f;
    p->cloud_top_offset = 1.0f;
    const float outer = R + 20000.0f;  // SUN_LOCATION and BACKGROUND_SKY_SUN_LOCATION
    p->sun_light_pos[1] = outer * 0.9f, p->sun_light_pos[2] = -outer * 0.9f;
    p->sky_sun_pos[1] = R * 2.0f, p->sky_sun_pos[2] = -R * 10.0f;
    p->eye_sign = -1.0f;  // the shader marches from -camera.eye
    p->feedback_min = 0.0f, p->feedback_max = 0.5f;
    for (int id = 0; id < 16; ++id) p->slot_x[id] = id / 4, p->slot_y[id] = id % 4;
    p->storage = MT_STORAGE_U8;
}

void orc_params_config(mt_params* p) {
    orc_params_reference(p);
    const float R = 6.36e6f;
    p->earth_radius = R;
    p->shell_inner_radius = R + 1500.0f, p->shell_outer_radius = R + 4000.0f;
    p->steps_min = p->steps_max = 128;
    p->accum_limit = 0.99f;  // transmittance below 0.01
    p->coverage_mode = 1, p->height_gradient = 1;
    const float h = 0.70710678f;  // heading 45 deg
    p->wind_dir[0] = h, p->wind_dir[1] = 0.0f, p->wind_dir[2] = h;
    p->wind_speed = 10.0f / ((p->shell_outer_radius - p->shell_inner_radius) * p->noise_period);
    p->skew_dir[0] = h, p->skew_dir[1] = 0.0f, p->skew_dir[2] = h;
    const float far = 1.0e9f;  // default sun 30 deg up toward -z (scenes set their own)
    p->sun_light_pos[0] = 0.0f, p->sun_light_pos[1] = 0.5f * far, p->sun_light_pos[2] = -0.86602540f * far;
    for (int i = 0; i < 3; ++i) p->sky_sun_pos[i] = p->sun_light_pos[i];
    p->eye_sign = 1.0f;
    p->feedback_min = p->feedback_max = 0.1f;  // history weight 0.9
    // 4x4 Bayer order: frame i marches the block position holding i
    static const int bayer[4][4] = {{0, 8, 2, 10}, {12, 4, 14, 6}, {3, 11, 1, 9}, {15, 7, 13, 5}};
    for (int y = 0; y < 4; ++y)
        for (int x = 0; x < 4; ++x) p->slot_x[bayer[y][x]] = x, p->slot_y[bayer[y][x]] = y;
}

}  // extern "C"
