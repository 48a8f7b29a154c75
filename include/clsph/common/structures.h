// Shared host/device data model of libclsph (libclsph/common/structures.h:16-54),
// declared without OpenCL headers: cl_float3 is a 16-byte union with .s[4]
// (and .x/.y/.z/.w), exactly the host layout of the reference's cl_float3, so
// `particle` is 80 bytes and `simulation_parameters` 128 bytes. These are the
// byte formats of the callbacks, of last_frame.bin and of the C ABI
// (include/clsph_gpu.h: clsph_particle, clsph_parameters, clsph_kernel_terms).
#ifndef _STRUCTURES_H_
#define _STRUCTURES_H_

#include <stdint.h>

#ifdef __cplusplus
// The reference's host-side structures.h reaches these through
// util/cl_boilerplate.h:4-8, and code written against it relies on them.
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>
#endif

typedef float cl_float;
typedef uint32_t cl_uint;
typedef int32_t cl_int;

typedef union {
  cl_float s[4];
  struct {
    cl_float x, y, z, w;
  };
} __attribute__((aligned(16))) cl_float3;

typedef union {
  cl_uint s[4];
  struct {
    cl_uint x, y, z, w;
  };
} __attribute__((aligned(16))) cl_uint3;

#define COLLISION_VOLUMES_COUNT 3

typedef struct {
  cl_uint particles_count;
  cl_float max_velocity;
  cl_float fluid_density;
  cl_float total_mass;
  cl_float particle_mass;
  cl_float dynamic_viscosity;
  cl_float simulation_time;
  cl_float target_fps;
  cl_float h;
  cl_float simulation_scale;
  cl_float time_delta;
  cl_float surface_tension_threshold;
  cl_float surface_tension;
  cl_float restitution;
  cl_float K;

  cl_float3 constant_acceleration;

  cl_int grid_size_x;
  cl_int grid_size_y;
  cl_int grid_size_z;
  cl_uint grid_cell_count;
  cl_float3 min_point, max_point;
} simulation_parameters;

typedef struct {
  cl_float3 position, velocity, intermediate_velocity, acceleration;
  cl_float density, pressure;
  cl_uint grid_index;
} particle;

typedef struct {
  float poly_6;
  float poly_6_gradient;
  float poly_6_laplacian;
  float spiky;
  float viscosity;
} precomputed_kernel_values;

#ifdef __cplusplus
static_assert(sizeof(particle) == 80, "particle must match the reference's 80-byte host layout");
static_assert(sizeof(simulation_parameters) == 128, "simulation_parameters must be 128 bytes");
static_assert(sizeof(precomputed_kernel_values) == 20, "precomputed_kernel_values must be 20 bytes");
#endif

#endif
