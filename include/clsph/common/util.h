// Morton (Z-curve) cell index helpers of libclsph/common/util.h:4-62: 10 bits
// per axis, x in bit 3k, y in bit 3k+1, z in bit 3k+2. Header-only (inline).
#ifndef _UTIL_H_
#define _UTIL_H_

#include "structures.h"

inline cl_uint clsph_spread10(cl_uint v) {
  v &= 0x3FFu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

// every third bit of `value`, starting at bit 0, packed into the low 10 bits
inline cl_uint uninterleave(cl_uint value) {
  cl_uint out = 0;
  for (int b = 0; b < 10; ++b) out |= ((value >> (3 * b)) & 1u) << b;
  return out;
}

inline cl_uint3 get_cell_coords_z_curve(cl_uint index) {
  cl_uint3 c;
  c.s[0] = uninterleave(index);
  c.s[1] = uninterleave(index >> 1);
  c.s[2] = uninterleave(index >> 2);
  c.s[3] = 0;
  return c;
}

inline cl_uint get_grid_index_z_curve(cl_uint x, cl_uint y, cl_uint z) {
  return clsph_spread10(x) | (clsph_spread10(y) << 1) | (clsph_spread10(z) << 2);
}

#endif
