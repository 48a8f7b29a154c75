// CPU oracle for the libclsph per-substep SPH path — TEST INFRASTRUCTURE.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// this library, and only as the oracle or the timed CPU baseline. The product
// (libclsph_gb300) never links or calls it.
//
// It restates, in its own code, what the reference computes for one substep:
//   bounding box + grid        libclsph/sph_simulation.cpp:199-252
//   Morton cell key            libclsph/common/util.h:4-62, kernels/grid.cl:43-67
//   stable sort + cell table   libclsph/sph_simulation.cpp:107-171, kernels/sort.cl:1-59
//   smoothing kernels          libclsph/kernels/smoothing.cl:1-34
//   density + Tait pressure    kernels/forces.cl:15-43, kernels/sph.cl:9-40
//   internal forces            kernels/forces.cl:45-112, kernels/sph.cl:42-62
//   leapfrog + mesh collision  kernels/advection.cl:6-23, kernels/collisions.cl:15-129,
//                              kernels/sph.cl:64-112
//   parameter derivation       libclsph/sph_simulation.cpp:490-505
//   initial lattice            libclsph/sph_simulation.cpp:48-94
//
// Single precision follows the reference's expression order operation by
// operation with plain IEEE float arithmetic (built with -ffp-contract=off),
// so it reproduces oracle/_ref bit for bit. The stable sort is a counting sort
// over the dense cell range, which yields the same permutation as the
// reference's 4-pass LSD radix sort and the cell table as its prefix sum.
// The same templates instantiated with double give the FP64 oracle.

#include "clsph_oracle.h"

#include <cmath>
#include <cstddef>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct alignas(16) F4 {
  float x, y, z, w;
};

// libclsph/common/structures.h:42-46 host layout (80 bytes)
struct Particle {
  F4 pos, vel, ivel, acc;
  float density, pressure;
  uint32_t key;
  uint32_t pad_;
};

// libclsph/common/structures.h:16-40 host layout (128 bytes)
struct Params {
  uint32_t n;
  float max_velocity, fluid_density, total_mass, particle_mass, dynamic_viscosity,
      simulation_time, target_fps, h, simulation_scale, time_delta, surface_tension_threshold,
      surface_tension, restitution, K;
  float pad_;
  F4 gravity;
  int32_t gx, gy, gz;
  uint32_t cell_count;
  F4 min_point, max_point;
};

struct Terms {
  float poly6, grad6, lap6, spiky, visc;
};

static_assert(sizeof(Particle) == 80, "particle layout");
static_assert(offsetof(Particle, density) == 64, "particle layout");
static_assert(offsetof(Particle, key) == 72, "particle layout");
static_assert(sizeof(Params) == 128, "parameter layout");
static_assert(offsetof(Params, gravity) == 64, "parameter layout");
static_assert(offsetof(Params, gx) == 80, "parameter layout");
static_assert(offsetof(Params, min_point) == 96, "parameter layout");

// ---------------------------------------------------------------- Morton keys
// 10 bits per axis, x in bit 3k, y in 3k+1, z in 3k+2 (util.h:41-62).
uint32_t spread10(uint32_t v) {
  uint32_t out = 0;
  for (int b = 0; b < 10; ++b) out |= ((v >> b) & 1u) << (3 * b);
  return out;
}
uint32_t gather10(uint32_t k) {
  uint32_t out = 0;
  for (int b = 0; b < 10; ++b) out |= ((k >> (3 * b)) & 1u) << b;
  return out;
}
uint32_t morton(uint32_t x, uint32_t y, uint32_t z) {
  return spread10(x) | (spread10(y) << 1) | (spread10(z) << 2);
}

// float -> uint cell coordinate. The reference casts a value that is >= 2 by
// construction (two padding cells); out-of-range values saturate here.
uint32_t cell_coord(float t) {
  if (!(t >= 0.f)) return 0u;
  if (t >= 4294967296.f) return 0xFFFFFFFFu;
  return (uint32_t)t;
}

// ------------------------------------------------------------- vector helpers
template <class T>
struct V3 {
  T x, y, z;
};
template <class T>
V3<T> sub(V3<T> a, V3<T> b) {
  return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <class T>
T norm(V3<T> v) {
  return std::sqrt((v.x * v.x + v.y * v.y) + v.z * v.z);
}
template <class T>
T dot3(V3<T> a, V3<T> b) {
  return (a.x * b.x + a.y * b.y) + a.z * b.z;
}
template <class T>
V3<T> ld(const F4& f) {
  return {(T)f.x, (T)f.y, (T)f.z};
}

// ---------------------------------------------------------- smoothing kernels
// smoothing.cl:1-34. `cut` is the (1 - clamp(floor(r/h), 0, 1)) support factor.
template <class T>
struct Kern {
  T h, poly6, grad6, lap6, spiky, visc, spiky_zero;
};

template <class T>
T cut(T r, T h) {
  T f = std::floor(r / h);
  f = f < T(0) ? T(0) : (f > T(1) ? T(1) : f);
  return T(1) - f;
}

template <class T>
T w_poly6(T r, const Kern<T>& k) {
  T d = k.h * k.h - r * r;
  return (cut(r, k.h) * k.poly6) * ((d * d) * d);
}

template <class T>
V3<T> grad_poly6(V3<T> rv, const Kern<T>& k) {
  T len = norm(rv);
  T d = k.h * k.h - len * len;
  T d2 = d * d;
  T s = cut(len, k.h) * k.grad6;
  return {(s * rv.x) * d2, (s * rv.y) * d2, (s * rv.z) * d2};
}

template <class T>
T lap_poly6(T r, const Kern<T>& k) {
  T a = std::fabs(r);
  return ((cut(a, k.h) * k.lap6) * (k.h * k.h - r * r)) * (T(3) * (k.h * k.h) - T(7) * (r * r));
}

template <class T>
V3<T> grad_spiky(V3<T> rv, const Kern<T>& k) {
  T len = norm(rv);
  if (len - T(0.0000001f) < T(0) && T(0) < len + T(0.0000001f))
    return {k.spiky_zero, k.spiky_zero, k.spiky_zero};  // smoothing.cl:23-25
  T s = cut(len, k.h) * k.spiky;
  T q = k.h - len;
  T q2 = q * q;
  return {(s * (rv.x / len)) * q2, (s * (rv.y / len)) * q2, (s * (rv.z / len)) * q2};
}

template <class T>
T lap_visc(T r, const Kern<T>& k) {
  return (cut(r, k.h) * k.visc) * (k.h - r);
}

template <class T>
T pow_n(T x, int n) {  // pown: n-1 left-to-right multiplies
  T r = x;
  for (int i = 1; i < n; ++i) r = r * x;
  return r;
}

Kern<float> kern_f32(const Params& p, const Terms& t) {
  Kern<float> k;
  k.h = p.h;
  k.poly6 = t.poly6;
  k.grad6 = t.grad6;
  k.lap6 = t.lap6;
  k.spiky = t.spiky;
  k.visc = t.visc;
  k.spiky_zero = -45.f / (float)(M_PI * (double)pow_n(p.h, 6));
  return k;
}

Kern<double> kern_f64(const Params& p) {
  Kern<double> k;
  double h = p.h;
  k.h = h;
  k.poly6 = 315.0 / (64.0 * M_PI * std::pow(h, 9.0));
  k.grad6 = -945.0 / (32.0 * M_PI * std::pow(h, 9.0));
  k.lap6 = k.grad6;
  k.spiky = -45.0 / (M_PI * std::pow(h, 6.0));
  k.visc = 45.0 / (M_PI * std::pow(h, 6.0));
  k.spiky_zero = k.spiky;
  return k;
}

// --------------------------------------------------------------- cell lookup
struct Grid {
  const uint32_t* table;
  uint32_t cells;
  uint32_t n;
  void range(uint32_t key, uint32_t& s, uint32_t& e) const {  // grid.cl:22-32
    if (key >= cells) {  // outside the dense table: treated as empty
      s = e = 0;
      return;
    }
    s = table[key];
    e = (cells > key + 1) ? table[key + 1] : n;
  }
};

// Visits the 27 cells in the reference's z, y, x order (forces.cl:25-27).
template <class F>
void for_each_candidate(uint32_t key, const Grid& g, F&& f) {
  uint32_t cx = gather10(key), cy = gather10(key >> 1), cz = gather10(key >> 2);
  for (uint32_t z = cz - 1; z <= cz + 1; ++z)
    for (uint32_t y = cy - 1; y <= cy + 1; ++y)
      for (uint32_t x = cx - 1; x <= cx + 1; ++x) {
        uint32_t s, e;
        g.range(morton(x, y, z), s, e);
        for (uint32_t j = s; j < e; ++j) f(j);
      }
}

// ------------------------------------------------------------ density (T)
template <class T>
T density_at(uint32_t i, const Particle* ps, const Grid& g, T mass, const Kern<T>& k) {
  T rho = T(0);
  V3<T> pi = ld<T>(ps[i].pos);
  for_each_candidate(ps[i].key, g, [&](uint32_t j) {
    T r = norm(sub(pi, ld<T>(ps[j].pos)));
    rho += mass * w_poly6(r, k);
  });
  return rho;
}

template <class T>
T tait(T rho, T rho0, T K) {
  return K * (pow_n(rho / rho0, 7) - T(1));
}

// -------------------------------------------------------------- forces (T)
// forces.cl:45-112 followed by sph.cl:53-58 (divide by density, add gravity).
template <class T>
V3<T> accel_at(uint32_t i, const Particle* ps, const T* rho, const T* prs, const Grid& g,
               const Params& p, const Kern<T>& k) {
  const T m = (T)p.particle_mass;
  V3<T> P{0, 0, 0}, Vs{0, 0, 0}, Nrm{0, 0, 0};
  T lap = T(0);
  const V3<T> pi = ld<T>(ps[i].pos);
  const V3<T> vi = ld<T>(ps[i].vel);
  const T own = prs[i] / (rho[i] * rho[i]);
  for_each_candidate(ps[i].key, g, [&](uint32_t j) {
    V3<T> rv = sub(pi, ld<T>(ps[j].pos));
    T mj = m / rho[j];
    if (j != i) {
      T coef = (prs[j] / (rho[j] * rho[j]) + own) * m;
      V3<T> sg = grad_spiky(rv, k);
      P.x += coef * sg.x;
      P.y += coef * sg.y;
      P.z += coef * sg.z;
      T vl = lap_visc(norm(rv), k);
      V3<T> dv = sub(ld<T>(ps[j].vel), vi);
      Vs.x += (dv.x * mj) * vl;
      Vs.y += (dv.y * mj) * vl;
      Vs.z += (dv.z * mj) * vl;
    }
    V3<T> g6 = grad_poly6(rv, k);
    Nrm.x += mj * g6.x;
    Nrm.y += mj * g6.y;
    Nrm.z += mj * g6.z;
    lap += mj * lap_poly6(norm(rv), k);
  });
  const T nrho = -rho[i];
  const T mu = (T)p.dynamic_viscosity;
  V3<T> sum{nrho * P.x + Vs.x * mu, nrho * P.y + Vs.y * mu, nrho * P.z + Vs.z * mu};
  T nlen = norm(Nrm);
  if (nlen > (T)p.surface_tension_threshold) {
    T s = -(T)p.surface_tension * lap;
    sum.x += (s * Nrm.x) / nlen;
    sum.y += (s * Nrm.y) / nlen;
    sum.z += (s * Nrm.z) / nlen;
  }
  return {sum.x / rho[i] + (T)p.gravity.x, sum.y / rho[i] + (T)p.gravity.y,
          sum.z / rho[i] + (T)p.gravity.z};
}

// ------------------------------------------------------ advection + collision
struct Hit {
  V3<float> point, normal;
  float depth;
  bool any;
};

// collisions.cl:15-89: nearest segment/triangle hit, an equal distance
// replaces the previous hit (later face wins).
bool nearest_hit(V3<float> p0, V3<float> p1, const float* fn, const float* vx,
                 const uint32_t* ix, uint32_t faces, Hit& h) {
  h.any = false;
  const V3<float> d = sub(p1, p0);
  for (uint32_t f = 0; f < faces; ++f) {
    V3<float> nrm{fn[3 * f], fn[3 * f + 1], fn[3 * f + 2]};
    if (dot3(nrm, d) / (norm(nrm) * norm(d)) <= 0.f) nrm = {-nrm.x, -nrm.y, -nrm.z};
    const uint32_t a = ix[3 * f], b = ix[3 * f + 1], c = ix[3 * f + 2];
    V3<float> v0{vx[3 * a], vx[3 * a + 1], vx[3 * a + 2]};
    V3<float> v1{vx[3 * b], vx[3 * b + 1], vx[3 * b + 2]};
    V3<float> v2{vx[3 * c], vx[3 * c + 1], vx[3 * c + 2]};
    V3<float> u = sub(v1, v0), v = sub(v2, v0);
    float den = dot3(nrm, d);
    if (den == 0.f) continue;
    float r = dot3(nrm, sub(v0, p0)) / den;
    if (!(0.f <= r && r <= 1.f)) continue;
    V3<float> at{p0.x + r * d.x, p0.y + r * d.y, p0.z + r * d.z};
    V3<float> w = sub(at, v0);
    float uv = dot3(u, v), wv = dot3(w, v), vv = dot3(v, v), wu = dot3(w, u), uu = dot3(u, u);
    float den2 = uv * uv - uu * vv;
    float s = (uv * wv - vv * wu) / den2;
    float t = (uv * wu - uu * wv) / den2;
    if (s >= 0.f && t >= 0.f && s + t <= 1.f) {
      if (h.any && norm(sub(p0, at)) > norm(sub(p0, h.point))) continue;
      h.normal = nrm;
      h.point = at;
      h.depth = norm(sub(p1, at));
      h.any = true;
    }
  }
  return h.any;
}

// sph.cl:64-112 with advection.cl:6-23 and collisions.cl:91-129.
bool advect_collide(Particle& q, const Params& p, const float* fn, const float* vx,
                    const uint32_t* ix, uint32_t faces, uint32_t max_iters) {
  float remaining = p.time_delta * p.simulation_scale;
  V3<float> pos = ld<float>(q.pos);
  V3<float> v = ld<float>(q.ivel);
  V3<float> a = ld<float>(q.acc);
  const V3<float> v_half_old = v;
  bool capped = false;
  for (uint32_t it = 0;; ++it) {
    // leapfrog with the speed clamp
    V3<float> nv{v.x + a.x * remaining, v.y + a.y * remaining, v.z + a.z * remaining};
    float sp = norm(nv);
    if (sp > p.max_velocity) {
      nv = {(nv.x / sp) * p.max_velocity, (nv.y / sp) * p.max_velocity,
            (nv.z / sp) * p.max_velocity};
    }
    V3<float> np{pos.x + nv.x * remaining, pos.y + nv.y * remaining, pos.z + nv.z * remaining};
    Hit h;
    bool hit = nearest_hit(pos, np, fn, vx, ix, faces, h);
    float elapsed = remaining;
    V3<float> out_pos = np;
    V3<float> out_v = nv;
    if (hit) {
      const float push = 0.001f;
      out_pos = {h.point.x - h.normal.x * push, h.point.y - h.normal.y * push,
                 h.point.z - h.normal.z * push};
      float k = (1.f + p.restitution * h.depth / (remaining * norm(nv))) * dot3(nv, h.normal);
      out_v = {nv.x - k * h.normal.x, nv.y - k * h.normal.y, nv.z - k * h.normal.z};
      elapsed = remaining * (norm(sub(out_pos, pos)) / norm(sub(np, pos)));
    }
    pos = out_pos;
    v = out_v;
    remaining -= elapsed;
    a = {0.f, 0.f, 0.f};
    if (!hit) break;
    if (it + 1 >= max_iters) {
      capped = true;
      break;
    }
  }
  q.vel = {(v_half_old.x + v.x) / 2.f, (v_half_old.y + v.y) / 2.f, (v_half_old.z + v.z) / 2.f,
           0.f};
  q.ivel = {v.x, v.y, v.z, 0.f};
  q.pos = {pos.x, pos.y, pos.z, 0.f};
  q.acc = {0.f, 0.f, 0.f, 0.f};
  return capped;
}

int resolve_threads(int threads) {
#ifdef _OPENMP
  return threads > 0 ? threads : omp_get_max_threads();
#else
  (void)threads;
  return 1;
#endif
}

// One substep; the body of clsph_oracle_step.
int step_impl(Params& p, const Terms& terms, const float* fn, const float* vx, const uint32_t* ix,
              uint32_t faces, Particle* host, uint32_t n, uint32_t* perm_out,
              std::vector<uint32_t>* table_out, void* snap_sorted, void* snap_density,
              void* snap_forces, uint32_t max_iters, uint32_t* capped_out, int threads) {
  p.n = n;
  const int nt = resolve_threads(threads);
  // bounding box (sph_simulation.cpp:199-217): `<`/`>` comparisons skip NaN
  const float cell = p.h * 2;
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = (float)std::numeric_limits<int>::max();
    hi[a] = (float)std::numeric_limits<int>::min();
  }
  for (uint32_t i = 0; i < n; ++i) {
    const float c[3] = {host[i].pos.x, host[i].pos.y, host[i].pos.z};
    for (int a = 0; a < 3; ++a) {
      if (c[a] < lo[a]) lo[a] = c[a];
      if (c[a] > hi[a]) hi[a] = c[a];
    }
  }
  for (int a = 0; a < 3; ++a) {
    lo[a] -= cell * 2;
    hi[a] += cell * 2;
  }
  p.min_point = {lo[0], lo[1], lo[2], 0.f};
  p.max_point = {hi[0], hi[1], hi[2], 0.f};
  p.gx = (int32_t)cell_coord((hi[0] - lo[0]) / cell);
  p.gy = (int32_t)cell_coord((hi[1] - lo[1]) / cell);
  p.gz = (int32_t)cell_coord((hi[2] - lo[2]) / cell);
  if (p.gx < 0 || p.gy < 0 || p.gz < 0 || p.gx >= 1024 || p.gy >= 1024 || p.gz >= 1024) return 2;
  p.cell_count = morton((uint32_t)p.gx, (uint32_t)p.gy, (uint32_t)p.gz);

  // keys (grid.cl:56-66)
  std::vector<uint32_t> key(n);
#pragma omp parallel for num_threads(nt) schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const Particle& q = host[i];
    key[i] = morton(cell_coord((q.pos.x - lo[0]) / (p.h * 2)),
                    cell_coord((q.pos.y - lo[1]) / (p.h * 2)),
                    cell_coord((q.pos.z - lo[2]) / (p.h * 2)));
  }

  // stable counting sort over the dense cell range; the exclusive prefix sum of
  // the counts is the reference's cell table (sph_simulation.cpp:162-170)
  std::vector<uint32_t> table((size_t)p.cell_count + 1, 0u);
  std::vector<uint32_t> perm(n);
  {
    std::vector<uint32_t> cursor((size_t)p.cell_count + 1, 0u);
    for (uint32_t i = 0; i < n; ++i)
      if (key[i] < p.cell_count) cursor[key[i]]++;
    uint32_t run = 0;
    for (size_t c = 0; c < p.cell_count; ++c) {
      uint32_t cnt = cursor[c];
      table[c] = run;
      cursor[c] = run;
      run += cnt;
    }
    table[p.cell_count] = run;
    // keys at or beyond the dense range (impossible with two padding cells)
    // go last, in input order
    cursor[p.cell_count] = run;
    for (uint32_t i = 0; i < n; ++i) {
      uint32_t b = key[i] < p.cell_count ? key[i] : p.cell_count;
      perm[cursor[b]++] = i;
    }
  }
  std::vector<Particle> sorted(n);
  for (uint32_t s = 0; s < n; ++s) {
    sorted[s] = host[perm[s]];
    sorted[s].key = key[perm[s]];
  }
  if (perm_out) std::memcpy(perm_out, perm.data(), sizeof(uint32_t) * n);
  if (snap_sorted) std::memcpy(snap_sorted, sorted.data(), sizeof(Particle) * n);
  table.resize(p.cell_count);
  if (table_out) *table_out = table;
  Grid g{table.data(), p.cell_count, n};

  // density + pressure
  const Kern<float> k = kern_f32(p, terms);
  std::vector<float> rho(n), prs(n);
#pragma omp parallel for num_threads(nt) schedule(dynamic, 512)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    rho[i] = density_at<float>((uint32_t)i, sorted.data(), g, p.particle_mass, k);
    prs[i] = tait<float>(rho[i], p.fluid_density, p.K);
  }
  for (uint32_t i = 0; i < n; ++i) {
    sorted[i].density = rho[i];
    sorted[i].pressure = prs[i];
  }
  if (snap_density) std::memcpy(snap_density, sorted.data(), sizeof(Particle) * n);

  // forces -> acceleration
  std::vector<V3<float>> acc(n);
#pragma omp parallel for num_threads(nt) schedule(dynamic, 512)
  for (int64_t i = 0; i < (int64_t)n; ++i)
    acc[i] = accel_at<float>((uint32_t)i, sorted.data(), rho.data(), prs.data(), g, p, k);
  for (uint32_t i = 0; i < n; ++i) sorted[i].acc = {acc[i].x, acc[i].y, acc[i].z, 0.f};
  if (snap_forces) std::memcpy(snap_forces, sorted.data(), sizeof(Particle) * n);

  // advection + collision
  uint32_t capped = 0;
  const uint32_t iters = max_iters ? max_iters : 1000000u;
#pragma omp parallel for num_threads(nt) schedule(dynamic, 256) reduction(+ : capped)
  for (int64_t i = 0; i < (int64_t)n; ++i)
    capped += advect_collide(sorted[i], p, fn, vx, ix, faces, iters) ? 1u : 0u;
  if (capped_out) *capped_out = capped;
  std::memcpy(host, sorted.data(), sizeof(Particle) * n);
  return 0;
}

}  // namespace

extern "C" {

int clsph_oracle_step(const void* params_in, void* params_out, const void* terms_in,
                      const float* face_normals, const float* vertices, const uint32_t* indices,
                      uint32_t face_count, void* particles_io, uint32_t n, uint32_t* perm_out,
                      uint32_t* cell_table_out, uint64_t cell_table_cap, void* snap_sorted,
                      void* snap_density, void* snap_forces, uint32_t max_collision_iters,
                      uint32_t* capped_out, int threads) {
  if (!params_in || !terms_in || !particles_io || n == 0) return 1;
  if (face_count && (!face_normals || !vertices || !indices)) return 1;
  Params p;
  std::memcpy(&p, params_in, sizeof(p));
  Terms t;
  std::memcpy(&t, terms_in, sizeof(t));
  std::vector<uint32_t> table;
  int rc = step_impl(p, t, face_normals, vertices, indices, face_count,
                     static_cast<Particle*>(particles_io), n, perm_out,
                     cell_table_out ? &table : nullptr, snap_sorted, snap_density, snap_forces,
                     max_collision_iters, capped_out, threads);
  if (rc == 2 && params_out) std::memcpy(params_out, &p, sizeof(p));
  if (rc) return rc;
  if (params_out) std::memcpy(params_out, &p, sizeof(p));
  if (cell_table_out) {
    if (cell_table_cap < table.size()) return 3;
    std::memcpy(cell_table_out, table.data(), sizeof(uint32_t) * table.size());
  }
  return 0;
}

int clsph_oracle_run(const void* params_in, const void* terms_in, const float* face_normals,
                     const float* vertices, const uint32_t* indices, uint32_t face_count,
                     void* particles_io, uint32_t n, uint32_t steps, int threads) {
  if (!params_in || !terms_in || !particles_io || n == 0) return 1;
  Params p;
  std::memcpy(&p, params_in, sizeof(p));
  Terms t;
  std::memcpy(&t, terms_in, sizeof(t));
  for (uint32_t s = 0; s < steps; ++s) {
    int rc = step_impl(p, t, face_normals, vertices, indices, face_count,
                       static_cast<Particle*>(particles_io), n, nullptr, nullptr, nullptr,
                       nullptr, nullptr, 1000000u, nullptr, threads);
    if (rc) return rc;
  }
  return 0;
}

int clsph_oracle_fields_f64(const void* params_in, const void* sorted_aos, uint32_t n,
                            const uint32_t* cell_table, double* density, double* pressure,
                            double* accel, int threads) {
  if (!params_in || !sorted_aos || !cell_table || !density || !pressure || !accel) return 1;
  Params p;
  std::memcpy(&p, params_in, sizeof(p));
  const Particle* ps = static_cast<const Particle*>(sorted_aos);
  const int nt = resolve_threads(threads);
  const Kern<double> k = kern_f64(p);
  Grid g{cell_table, p.cell_count, n};
#pragma omp parallel for num_threads(nt) schedule(dynamic, 512)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    density[i] = density_at<double>((uint32_t)i, ps, g, (double)p.particle_mass, k);
    pressure[i] = tait<double>(density[i], (double)p.fluid_density, (double)p.K);
  }
#pragma omp parallel for num_threads(nt) schedule(dynamic, 512)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    V3<double> a = accel_at<double>((uint32_t)i, ps, density, pressure, g, p, k);
    accel[3 * i] = a.x;
    accel[3 * i + 1] = a.y;
    accel[3 * i + 2] = a.z;
  }
  return 0;
}

void clsph_oracle_derive(void* params_io, void* terms_out, int influence_count,
                         float* initial_volume_out) {
  Params p;
  std::memcpy(&p, params_io, sizeof(p));
  Terms t;
  p.total_mass = p.n * p.particle_mass;
  const float volume = p.total_mass / p.fluid_density;
  // float arithmetic up to the division by the double 4*pi, then narrowed
  const double q = (3.f * (influence_count * (volume / p.n))) / (4.f * M_PI);
  p.h = std::cbrt((float)q);
  p.time_delta = 1.f / p.target_fps;
  p.max_velocity = 0.8f * p.h / p.time_delta;
  // the constants use the double overload of pow (plain ::pow on a float)
  const double h = p.h;
  t.poly6 = (float)(315.f / (64.f * M_PI * std::pow(h, 9.0)));
  t.grad6 = (float)(-945.f / (32.f * M_PI * std::pow(h, 9.0)));
  t.lap6 = (float)(-945.f / (32.f * M_PI * std::pow(h, 9.0)));
  t.spiky = (float)(-45.f / (M_PI * std::pow(h, 6.0)));
  t.visc = (float)(45.f / (M_PI * std::pow(h, 6.0)));
  std::memcpy(params_io, &p, sizeof(p));
  std::memcpy(terms_out, &t, sizeof(t));
  if (initial_volume_out) *initial_volume_out = volume;
}

void clsph_oracle_init_lattice(void* particles_out, uint32_t n, float initial_volume) {
  Particle* ps = static_cast<Particle*>(particles_out);
  const int side = (int)std::ceil(std::cbrt((float)n));
  const float len = std::cbrt(initial_volume);
  const float gap = len / (float)side;
  for (uint32_t i = 0; i < n; ++i) {
    Particle q;
    std::memset(&q, 0, sizeof(q));
    q.pos.x = (float)(i % side) * gap - len / 2.f;
    q.pos.y = (float)((i / side) % side) * gap;
    q.pos.z = (float)(i / (side * side)) * gap - len / 2.f;
    ps[i] = q;
  }
}

uint32_t clsph_oracle_morton(uint32_t x, uint32_t y, uint32_t z) { return morton(x, y, z); }

void clsph_oracle_cell_coords(uint32_t key, uint32_t* xyz) {
  xyz[0] = gather10(key);
  xyz[1] = gather10(key >> 1);
  xyz[2] = gather10(key >> 2);
}

}  // extern "C"
