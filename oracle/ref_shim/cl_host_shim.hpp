// OpenCL-C-as-host-C++ shim used ONLY to build oracle/_ref: it lets the
// reference's own kernel sources (libclsph/kernels/{smoothing,forces,grid,
// advection,collisions}.cl and libclsph/common/{structures,util}.h) compile
// unchanged as C++ so that the oracle restatement can be checked against them.
//
// This file is test infrastructure. It defines the OpenCL built-ins those
// sources use with plain IEEE single-precision arithmetic (no FMA contraction;
// build with -ffp-contract=off). OpenCL itself leaves the accuracy of
// length/distance/normalize/pown implementation-defined; the definitions here
// are the ones the whole project treats as "the reference's FP32 results":
//   length(v)    = sqrt((x*x + y*y) + z*z);  length(scalar) = |scalar|
//   dot(a,b)     = (ax*bx + ay*by) + az*bz
//   distance     = length(a - b)
//   normalize(v) = v / length(v)          (component-wise divide)
//   pown(x, n)   = ((x*x)*x)...           (n-1 left-to-right multiplies)
//   float3 * double scalar: the scalar is narrowed to float first, as OpenCL
//   does for a vector/scalar mix.
//
// The shim must be included inside a namespace (see ref_driver.cpp) so that
// its floor/clamp/length overloads do not collide with <cmath>.

#ifndef CLSPH_CL_HOST_SHIM_HPP
#define CLSPH_CL_HOST_SHIM_HPP

// address-space and function qualifiers vanish on the host
#define global
#define __global
#define constant const
#define kernel
#define __kernel

typedef unsigned int uint;

// OpenCL float3 occupies 16 bytes (same as cl_float3 = cl_float4 on the host).
struct alignas(16) float3 {
  float x, y, z, w;
  float3() : x(0.f), y(0.f), z(0.f), w(0.f) {}
  float3(float s) : x(s), y(s), z(s), w(0.f) {}  // scalar broadcast
  float3(float a, float b, float c) : x(a), y(b), z(c), w(0.f) {}
};

struct alignas(16) uint3 {
  uint x, y, z, w;
  uint3() : x(0), y(0), z(0), w(0) {}
  uint3(uint a, uint b, uint c) : x(a), y(b), z(c), w(0) {}
};

struct alignas(8) uint2 {
  uint x, y;
  uint2() : x(0), y(0) {}
  uint2(uint a, uint b) : x(a), y(b) {}
};

inline float3 operator+(float3 a, float3 b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(float3 a, float3 b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator*(float3 a, float3 b) { return float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator-(float3 a) { return float3(-a.x, -a.y, -a.z); }
inline float3 operator*(float3 a, float s) { return float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator*(float s, float3 a) { return float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator*(float3 a, double s) { return a * (float)s; }
inline float3 operator*(double s, float3 a) { return (float)s * a; }
inline float3 operator/(float3 a, float s) { return float3(a.x / s, a.y / s, a.z / s); }
inline float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
inline float3& operator-=(float3& a, float3 b) { a = a - b; return a; }

inline float dot(float3 a, float3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(float3 v) { return std::sqrt((v.x * v.x + v.y * v.y) + v.z * v.z); }
// OpenCL's scalar length() is |x| (smoothing.cl:14 applies it to a float).
inline float length(float x) { return std::fabs(x); }
inline float distance(float3 a, float3 b) { return length(a - b); }
inline float3 normalize(float3 v) { float l = length(v); return v / l; }

inline float pown(float x, int n) {
  if (n == 0) return 1.f;
  float r = x;
  for (int i = 1; i < n; ++i) r = r * x;
  return r;
}
inline float floor(float x) { return std::floor(x); }
inline float clamp(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }
inline float convert_float(float x) { return x; }
inline float convert_float(double x) { return (float)x; }

#endif
