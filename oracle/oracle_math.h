// CPU restatement of prender's radiance estimator — TEST INFRASTRUCTURE ONLY.
//
// This directory is the oracle: a plain C++ restatement of the reference
// algorithm that the GPU path is checked against.  Only tests/, the smoke
// check and bench.py's CPU-baseline leg may load it.  It is never part of
// the product path.
//
// oracle_math.h: FP64 vector arithmetic with the reference's exact
// operation order, and MT19937-64.  Compiled with -ffp-contract=off so that
// results are identical on x86-64 and AArch64.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>

namespace orc {

constexpr double PI = 3.14159265358979323846264338327950288;       // constant.h:5
constexpr double TWOPI = 6.28318530717958647692528676655900576;    // constant.h:19
constexpr double INV_PI = 0.31830988618379067153776752674502872;   // constant.h:9
constexpr double FORPI = 12.5663706143591729538505735331180115;    // constant.h:24
constexpr double INV_FORPI = 0.07957747154594766788444188168625718;// constant.h:26
constexpr double RAD = PI / 180.0;                                 // constant.h:31 (PS_RAD)
constexpr double INF = 1.0e128;                                    // constant.h:33
constexpr double EPS = 1.0e-6;                                     // constant.h:36
constexpr double EPS14 = 1.0e-14;                                  // constant.h:39
constexpr double EPS12 = 1.0e-12;
constexpr double EPS16 = 1.0e-16;

struct V3 {
  double x = 0, y = 0, z = 0;
  V3() = default;
  V3(double a, double b, double c) : x(a), y(b), z(c) {}
  explicit V3(double a) : x(a), y(a), z(a) {}
  double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, double b) { return {a.x * b, a.y * b, a.z * b}; }
inline V3 operator*(double b, V3 a) { return {b * a.x, b * a.y, b * a.z}; }
// component-wise product (vector3d.h multiply)
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
// Vector3d::operator/(double) (vector3d.h): division by zero yields (1,1,1)
inline V3 operator/(V3 a, double b) {
  if (b == 0.0) return {1, 1, 1};
  return {a.x / b, a.y / b, a.z / b};
}
// The reference's SSE dot/sqr add the x,z lanes first, then y
// (vector3d.h USE_SIMD branch of dot() and sqr()).
inline double dot(V3 a, V3 b) { return (a.x * b.x + a.z * b.z) + a.y * b.y; }
inline double sqr(V3 a) { return (a.x * a.x + a.z * a.z) + a.y * a.y; }
inline double length(V3 a) { return std::sqrt(sqr(a)); }
inline V3 normalize(V3 a) { return a * (1.0 / length(a)); }
inline V3 cross(V3 a, V3 b) {
  return {(a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x)};
}
inline V3 vexp(V3 a) { return {std::exp(a.x), std::exp(a.y), std::exp(a.z)}; }

// OrthonormalBasis (vector3d.h:244-253)
inline void onb(V3 n, V3& w, V3& u, V3& v) {
  w = n;
  if (std::fabs(w.x) > EPS) u = normalize(cross(V3(0.0, 1.0, 0.0), w));
  else u = normalize(cross(V3(1.0, 0.0, 0.0), w));
  v = normalize(cross(w, u));
}

// The Random interface radiance() draws from (random.h:16-23): a stream
// generator, or the Metropolis sampler's primary samples (mlt.h:86-168).
struct Sampler {
  virtual double next01() = 0;
  // Random::Next01: the stream itself even under MLT (KelemenMLT::Next01,
  // mlt.h:166), which the light choice and the surface NEE point draw from
  virtual double Next01() { return next01(); }
  virtual ~Sampler() {}
};

// MT19937-64 (Matsumoto & Nishimura), the generator behind the reference's
// MTRandom (random.h:73-186, random.cpp:204-311); next01 is genrand64_real1.
struct MT64 : Sampler {
  static constexpr int NN = 312, MM = 156;
  uint64_t mt[NN];
  int mti = NN + 1;
  explicit MT64(uint64_t seed) { init(seed); }
  void init(uint64_t seed) {
    mt[0] = seed;
    for (mti = 1; mti < NN; mti++)
      mt[mti] = 6364136223846793005ULL * (mt[mti - 1] ^ (mt[mti - 1] >> 62)) + (uint64_t)mti;
  }
  uint64_t next_u64() {
    static const uint64_t mag01[2] = {0ULL, 0xB5026F5AA96619E9ULL};
    const uint64_t UM = 0xFFFFFFFF80000000ULL, LM = 0x7FFFFFFFULL;
    uint64_t x;
    if (mti >= NN) {
      int i;
      for (i = 0; i < NN - MM; i++) {
        x = (mt[i] & UM) | (mt[i + 1] & LM);
        mt[i] = mt[i + MM] ^ (x >> 1) ^ mag01[(int)(x & 1ULL)];
      }
      for (; i < NN - 1; i++) {
        x = (mt[i] & UM) | (mt[i + 1] & LM);
        mt[i] = mt[i + (MM - NN)] ^ (x >> 1) ^ mag01[(int)(x & 1ULL)];
      }
      x = (mt[NN - 1] & UM) | (mt[0] & LM);
      mt[NN - 1] = mt[MM - 1] ^ (x >> 1) ^ mag01[(int)(x & 1ULL)];
      mti = 0;
    }
    x = mt[mti++];
    x ^= (x >> 29) & 0x5555555555555555ULL;
    x ^= (x << 17) & 0x71D67FFFEDA60000ULL;
    x ^= (x << 37) & 0xFFF7EEE000000000ULL;
    x ^= (x >> 43);
    return x;
  }
  double next01() override { return (double)(next_u64() >> 11) * (1.0 / 9007199254740991.0); }
};

}  // namespace orc
