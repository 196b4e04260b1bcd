// Minimal .npy / .npz (uncompressed, as numpy.savez writes) reader and .npy writer for
// the command-line tool and the learned-octree weights.  Arrays are little-endian,
// C-ordered; supported element types: f4, f8, i4, i8, u4, u1, b1, c8.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace bpgb {

struct NpyArray {
    std::string descr;            // e.g. "<f4"
    std::vector<uint64_t> shape;  // empty for a scalar
    std::vector<unsigned char> bytes;
    uint64_t count() const;
    uint32_t itemsize() const;
    // Element i converted to double (complex: the real part) / the whole array as float.
    double at(uint64_t i) const;
    std::vector<float> as_float() const;
};

// Parses one .npy image; false with *why on a format it does not handle.
bool npy_parse(const unsigned char *data, size_t size, NpyArray *out, std::string *why);
bool npy_load(const std::string &path, NpyArray *out, std::string *why);
// Every member of an uncompressed .npz ("name.npy" entries, keys without ".npy");
// members of other element types (text, objects) are skipped.
bool npz_load(const std::string &path, std::map<std::string, NpyArray> *out, std::string *why);
// Writes a float32 C-ordered .npy (version 1.0 header).
bool npy_save_f32(const std::string &path, const float *data, const std::vector<uint64_t> &shape,
                  std::string *why);

}  // namespace bpgb
