// TEST INFRASTRUCTURE — the oracle.  Not part of the product: only tests/ and
// the measurement scripts beside the oracle load it, and only to count work.
//
// An op-counting build of the raymarch restatement (oracle/meteoros_oracle.cpp):
// the restatement's templates instantiated on a float type that counts every
// +, -, *, / and every sqrt, exp, pow, acos and cos as one floating-point
// operation (comparisons, min/max, floor, abs and conversions count nothing).
// The arithmetic itself is plain FP32, so control flow and the sample counters
// equal the float oracle's.  orc_count_flops marches a list of pixels and
// returns, per ray, its operation count and its executed primary and light
// samples; oracle/count_flops.py fits FLOPs = a*rays + b*primary + c*light.
#include <cmath>
#include <cstdint>

namespace orc {

inline thread_local unsigned long long g_flops = 0;

struct CF {
    float v;
    CF() = default;
    constexpr CF(float x) : v(x) {}
    constexpr CF(double x) : v((float)x) {}
    constexpr CF(int x) : v((float)x) {}
    constexpr CF(unsigned x) : v((float)x) {}
    constexpr CF(long long x) : v((float)x) {}
    constexpr CF(unsigned char x) : v((float)x) {}
    explicit operator float() const { return v; }
    explicit operator double() const { return (double)v; }
};

inline CF operator+(CF a, CF b) { ++g_flops; return CF(a.v + b.v); }
inline CF operator-(CF a, CF b) { ++g_flops; return CF(a.v - b.v); }
inline CF operator*(CF a, CF b) { ++g_flops; return CF(a.v * b.v); }
inline CF operator/(CF a, CF b) { ++g_flops; return CF(a.v / b.v); }
inline CF operator-(CF a) { return CF(-a.v); }
inline CF& operator+=(CF& a, CF b) { return a = a + b; }
inline CF& operator-=(CF& a, CF b) { return a = a - b; }
inline CF& operator*=(CF& a, CF b) { return a = a * b; }
inline CF& operator/=(CF& a, CF b) { return a = a / b; }
inline bool operator<(CF a, CF b) { return a.v < b.v; }
inline bool operator>(CF a, CF b) { return a.v > b.v; }
inline bool operator<=(CF a, CF b) { return a.v <= b.v; }
inline bool operator>=(CF a, CF b) { return a.v >= b.v; }
inline bool operator==(CF a, CF b) { return a.v == b.v; }
inline bool operator!=(CF a, CF b) { return a.v != b.v; }

}  // namespace orc

namespace std {
inline orc::CF floor(orc::CF x) { return orc::CF(std::floor(x.v)); }
inline orc::CF fabs(orc::CF x) { return orc::CF(std::fabs(x.v)); }
inline orc::CF round(orc::CF x) { return orc::CF(std::round(x.v)); }
inline orc::CF sqrt(orc::CF x) { ++orc::g_flops; return orc::CF(std::sqrt(x.v)); }
inline orc::CF exp(orc::CF x) { ++orc::g_flops; return orc::CF(std::exp(x.v)); }
inline orc::CF pow(orc::CF x, orc::CF y) { ++orc::g_flops; return orc::CF(std::pow(x.v, y.v)); }
inline orc::CF acos(orc::CF x) { ++orc::g_flops; return orc::CF(std::acos(x.v)); }
inline orc::CF cos(orc::CF x) { ++orc::g_flops; return orc::CF(std::cos(x.v)); }
}  // namespace std

#include "oracle_math.hpp"

namespace orc {
inline int f2i(CF x) { return f2i((double)x.v); }
template <> constexpr CF lit<CF>(float f, double) { return CF(f); }
}  // namespace orc

#include "meteoros_oracle.cpp"

extern "C" {

// Marches the listed pixels (x, y pairs) as a full-raymarch frame would, one
// thread; per pixel writes {operations, primary samples, light samples, rays}.
__attribute__((visibility("default"))) int orc_count_flops(const orc_volumes* v, const mt_camera_ubo* cam,
                                                           const mt_time_ubo* tm, const mt_params* p, int W, int H,
                                                           const int32_t* xy, long long n, uint64_t* out) {
    if (!v || !cam || !tm || !p || !xy || !out || W <= 0 || H <= 0 || n < 0) return 1;
    orc::Frame<orc::CF> F = orc::make_frame<orc::CF>(v, cam, cam, tm, p);
    for (long long i = 0; i < n; ++i) {
        orc::Counters cnt;
        orc::CF m;
        orc::g_flops = 0;
        orc::march_pixel(F, xy[2 * i], xy[2 * i + 1], W, H, &m, cnt);
        out[4 * i] = orc::g_flops;
        out[4 * i + 1] = cnt.primary;
        out[4 * i + 2] = cnt.light;
        out[4 * i + 3] = cnt.rays;
    }
    return 0;
}

}  // extern "C"
