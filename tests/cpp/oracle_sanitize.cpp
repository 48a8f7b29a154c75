// Runs the CPU oracle (oracle/clsph_oracle.cpp) for a few substeps with every
// optional output enabled, for a build with AddressSanitizer and
// UndefinedBehaviorSanitizer. Inputs are raw files written by the test:
//   <dir>/params.bin (128 B)  terms.bin (20 B)  particles.bin (n x 80 B)
//   normals.bin, vertices.bin (float32)  indices.bin (uint32)
// Output: <dir>/out.bin, the particles after `steps` substeps.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iterator>
#include <vector>

#include "clsph_oracle.h"

static std::vector<char> slurp(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  return std::vector<char>(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s <dir> <steps>\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1];
  const int steps = std::atoi(argv[2]);
  std::vector<char> params = slurp(dir + "/params.bin"), terms = slurp(dir + "/terms.bin");
  std::vector<char> parts = slurp(dir + "/particles.bin");
  std::vector<char> normals = slurp(dir + "/normals.bin"), verts = slurp(dir + "/vertices.bin");
  std::vector<char> idx = slurp(dir + "/indices.bin");
  if (params.size() != 128 || terms.size() != 20 || parts.size() % 80 != 0) return 3;
  const uint32_t n = (uint32_t)(parts.size() / 80);
  const uint32_t faces = (uint32_t)(idx.size() / 12);
  std::vector<char> params_out(128), snap_a(parts.size()), snap_b(parts.size()), snap_c(parts.size());
  std::vector<uint32_t> perm(n);
  std::vector<uint32_t> table(1u << 16);  // grids of up to 2^16 Morton cells (16^3)
  for (int s = 0; s < steps; ++s) {
    uint32_t capped = 0;
    int rc = clsph_oracle_step(params.data(), params_out.data(), terms.data(),
                               (const float*)normals.data(), (const float*)verts.data(),
                               (const uint32_t*)idx.data(), faces, parts.data(), n, perm.data(),
                               table.data(), table.size(), snap_a.data(), snap_b.data(),
                               snap_c.data(), 0, &capped, 2);
    if (rc != 0) {
      std::fprintf(stderr, "clsph_oracle_step: status %d at substep %d\n", rc, s);
      return 4;
    }
    if (s == steps - 1) {
      std::vector<double> rho(n), prs(n), acc(3 * (size_t)n);
      rc = clsph_oracle_fields_f64(params_out.data(), snap_a.data(), n, table.data(), rho.data(),
                                   prs.data(), acc.data(), 2);
      if (rc != 0) return 5;
    }
  }
  std::ofstream out(dir + "/out.bin", std::ios::binary);
  out.write(parts.data(), (std::streamsize)parts.size());
  return 0;
}
