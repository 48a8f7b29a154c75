// Raw binary archives with the two calls libclsph uses for last_frame.bin
// (example/particles.cpp:40-44 saveBinary, sph_simulation.cpp:60-67
// loadBinary): the bytes of the particle AoS, no header. A minimal stand-in
// for the vendored cereal binary archive so that code written against the
// reference compiles unchanged.
#ifndef CLSPH_CEREAL_BINARY_HPP
#define CLSPH_CEREAL_BINARY_HPP

#include <cstddef>
#include <istream>
#include <ostream>
#include <stdexcept>

namespace cereal {

class BinaryOutputArchive {
 public:
  explicit BinaryOutputArchive(std::ostream& stream) : stream_(stream) {}
  void saveBinary(const void* data, std::size_t size) {
    stream_.write(static_cast<const char*>(data), static_cast<std::streamsize>(size));
    if (!stream_) throw std::runtime_error("Failed to write " + std::to_string(size) + " bytes to output stream!");
  }

 private:
  std::ostream& stream_;
};

class BinaryInputArchive {
 public:
  explicit BinaryInputArchive(std::istream& stream) : stream_(stream) {}
  void loadBinary(void* data, std::size_t size) {
    stream_.read(static_cast<char*>(data), static_cast<std::streamsize>(size));
    if (static_cast<std::size_t>(stream_.gcount()) != size)
      throw std::runtime_error("Failed to read " + std::to_string(size) + " bytes from input stream!");
  }

 private:
  std::istream& stream_;
};

}  // namespace cereal

#endif
