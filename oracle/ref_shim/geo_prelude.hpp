// TEST INFRASTRUCTURE (oracle/_ref only): host-side stand-ins for the OpenCL
// vector types that libclsph/common/structures.h names when it is compiled
// with KERNEL_INCLUDE (the reference's host build takes them from the OpenCL
// headers, which this machine lacks). cl_float3 is cl_float4 on the host: 16
// bytes, 16-byte aligned, components in .s[]. Also the stream headers the
// reference's houdini_file_saver.cpp receives through its OpenCL boilerplate
// header.
#pragma once

#include <fstream>
#include <iostream>

struct alignas(16) float3 {
  float s[4];
};
struct alignas(16) uint3 {
  unsigned int s[4];
};
