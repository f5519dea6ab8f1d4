// Host-side uniform producers and parameter presets of the C ABI
// (include/meteoros.h).  No GPU work happens here.
//
//   mt_time_init / mt_time_advance  <- Scene::InitializeTime / UpdateTime
//                                      (Scene.cpp:65-119)
//   mt_halton                       <- Scene::HaltonSequenceAt (Scene.cpp:125-138)
//   mt_camera_look_at               <- Camera::UpdateBuffer (camera.cpp:31-42),
//                                      Camera::GetView/GetProj (camera.cpp:56-63)
//   mt_params_reference             <- the #defines and literals of
//                                      cloudRayMarch.comp, reprojection.comp and
//                                      postProcess_TXAA.frag
//   mt_params_config                <- the physically parameterised presets
#include <cmath>
#include <cstring>

#include "../../include/meteoros.h"

namespace {

struct v3 {
    float x, y, z;
};
inline v3 sub(v3 a, v3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline v3 cross(v3 a, v3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
// glm::normalize: v * inversesqrt(dot(v, v)) with inversesqrt(x) = 1 / sqrt(x)
inline v3 normalize(v3 a) {
    const float inv = 1.0f / std::sqrt(dot(a, a));
    return {a.x * inv, a.y * inv, a.z * inv};
}

// 4x4 Bayer matrix: the slot of frame i is the position holding i.
const int kBayer4[4][4] = {{0, 8, 2, 10}, {12, 4, 14, 6}, {3, 11, 1, 9}, {15, 7, 13, 5}};

}  // namespace

extern "C" {

MT_API int mt_abi_version(void) { return MT_ABI_VERSION; }

MT_API float mt_halton(int index, int base) {
    float f = 1.0f;
    float r = 0.0f;
    while (index > 0) {
        f = f / (float)base;
        r += f * (float)(index % base);
        index = index / base;
    }
    return r;
}

MT_API void mt_time_init(mt_time_ubo* t) {
    if (!t) return;
    std::memset(t, 0, sizeof(*t));
    for (int i = 0; i < 4; ++i) {
        t->halton_seq1[i] = mt_halton(1 + i, 3);
        t->halton_seq2[i] = mt_halton(5 + i, 3);
        t->halton_seq3[i] = mt_halton(9 + i, 3);
        t->halton_seq4[i] = mt_halton(13 + i, 3);
    }
    t->frame_count_mod16 = 0;
}

MT_API void mt_time_advance(mt_time_ubo* t, float dt) {
    if (!t) return;
    t->time[0] = dt;
    t->time[1] += dt;
    t->frame_count_mod16 = (t->frame_count_mod16 + 1) % 16;
}

MT_API void mt_camera_look_at(mt_camera_ubo* out, const float eye[3], const float ref[3], float fovy_deg,
                              float aspect, float near_clip, float far_clip) {
    if (!out || !eye || !ref) return;
    std::memset(out, 0, sizeof(*out));
    const v3 e{eye[0], eye[1], eye[2]}, c{ref[0], ref[1], ref[2]};
    const v3 worldUp{0.0f, 1.0f, 0.0f};
    // Camera::RecomputeAttributes (camera.cpp:67-76)
    v3 forward = normalize(sub(c, e));
    v3 right = normalize(cross(forward, worldUp));
    v3 up = cross(right, forward);
    // lookAt(eye, ref, up), right-handed: rows s, u, -f; translation -dot.
    v3 f = normalize(sub(c, e));
    v3 s = normalize(cross(f, up));
    v3 u = cross(s, f);
    float* V = out->view;  // column-major: V[col*4 + row]
    V[0] = s.x;  V[4] = s.y;  V[8] = s.z;
    V[1] = u.x;  V[5] = u.y;  V[9] = u.z;
    V[2] = -f.x; V[6] = -f.y; V[10] = -f.z;
    V[12] = -dot(s, e);
    V[13] = -dot(u, e);
    V[14] = dot(f, e);
    V[15] = 1.0f;
    // perspective, right-handed, depth 0..1 (camera.h defines
    // GLM_FORCE_DEPTH_ZERO_TO_ONE), then proj[1][1] *= -1 (camera.cpp:35).
    const float rad = fovy_deg * (3.14159265358979323846f / 180.0f);
    const float th = std::tan(rad / 2.0f);
    float* P = out->proj;
    P[0] = 1.0f / (aspect * th);
    P[5] = -(1.0f / th);
    P[10] = far_clip / (near_clip - far_clip);
    P[11] = -1.0f;
    P[14] = -(far_clip * near_clip) / (far_clip - near_clip);
    out->eye[0] = eye[0];
    out->eye[1] = eye[1];
    out->eye[2] = eye[2];
    out->eye[3] = 1.0f;
    // camera.cpp:38-39 (PI there is 3.14159, evaluated in double)
    out->tan_fov_by_2[1] = (float)std::fabs(std::tan(fovy_deg * 0.5 * (3.14159 / 180.0)));
    out->tan_fov_by_2[0] = aspect * out->tan_fov_by_2[1];
}

MT_API void mt_params_reference(mt_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    const float R = 6371000.0f;
    p->earth_radius = R;
    p->shell_inner_radius = R + 7500.0f;
    p->shell_outer_radius = R + 20000.0f;
    p->noise_period = 8.0f;
    p->steps_min = 35;
    p->steps_max = 60;
    p->accum_limit = 1.0f;
    p->coverage_mode = 0;
    p->coverage = 0.6f;
    p->height_gradient = 0;
    p->weather_scale = 60000.0f;
    p->weather_slot = 0;
    p->wind_dir[0] = 1.0f + 0.0f;
    p->wind_dir[1] = 0.0f + 0.1f;
    p->wind_dir[2] = 0.0f + 0.0f;
    p->wind_speed = 0.080f;
    p->skew_dir[0] = 1.0f;
    p->skew_dir[1] = 0.0f;
    p->skew_dir[2] = 0.0f;
    p->cloud_top_offset = 1.0f;
    const float outer = R + 20000.0f;
    p->sun_light_pos[0] = 0.0f;
    p->sun_light_pos[1] = outer * 0.9f;
    p->sun_light_pos[2] = -outer * 0.9f;
    p->sky_sun_pos[0] = 0.0f;
    p->sky_sun_pos[1] = R * 2.0f;
    p->sky_sun_pos[2] = -R * 10.0f;
    p->eye_sign = -1.0f;
    p->feedback_min = 0.0f;
    p->feedback_max = 0.5f;
    for (int i = 0; i < 16; ++i) {
        // cloudRayMarch.comp:697-698: pX = int(floor(id/4)), pY = int(floor(mod(id,4)))
        p->slot_x[i] = (int)std::floor((float)(i / 4));
        const float fi = (float)i;
        p->slot_y[i] = (int)std::floor(fi - 4.0f * std::floor(fi / 4.0f));
    }
    p->storage = MT_STORAGE_U8;
    p->fp64_shells = 0;
}

MT_API void mt_params_config(mt_params* p) {
    if (!p) return;
    mt_params_reference(p);
    const float R = 6.36e6f;
    p->earth_radius = R;
    p->shell_inner_radius = R + 1500.0f;
    p->shell_outer_radius = R + 4000.0f;
    p->noise_period = 8.0f;
    p->steps_min = 128;
    p->steps_max = 128;
    p->accum_limit = 0.99f;  // transmittance 1 - accumulated density < 0.01
    p->coverage_mode = 1;
    p->height_gradient = 1;
    p->weather_scale = 60000.0f;
    // Wind 10 m/s at heading 45 deg, in noise units: metres / (thickness * noise_period).
    const float c45 = 0.70710678f;
    p->wind_dir[0] = c45;
    p->wind_dir[1] = 0.0f;
    p->wind_dir[2] = c45;
    p->wind_speed = 10.0f / ((p->shell_outer_radius - p->shell_inner_radius) * p->noise_period);
    p->skew_dir[0] = c45;
    p->skew_dir[1] = 0.0f;
    p->skew_dir[2] = c45;
    p->cloud_top_offset = 1.0f;
    // Default sun: elevation 30 deg toward -z; scenes override it.
    const float se = 0.5f, ce = 0.86602540f;
    const float far = 1.0e9f;
    p->sun_light_pos[0] = 0.0f;
    p->sun_light_pos[1] = se * far;
    p->sun_light_pos[2] = -ce * far;
    p->sky_sun_pos[0] = 0.0f;
    p->sky_sun_pos[1] = se * far;
    p->sky_sun_pos[2] = -ce * far;
    p->eye_sign = 1.0f;
    p->feedback_min = 0.1f;  // history weight 0.9
    p->feedback_max = 0.1f;
    for (int y = 0; y < 4; ++y)
        for (int x = 0; x < 4; ++x) {
            p->slot_x[kBayer4[y][x]] = x;
            p->slot_y[kBayer4[y][x]] = y;
        }
}

}  // extern "C"
