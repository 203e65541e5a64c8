// Binary little-endian .ply files: the header model shared by the 3D Gaussian
// Splatting reader and writer (src/plyLoader.ts, src/plyWriter.ts) and the
// trainer's checkpoints.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "dg_common.cuh"

namespace dg {

enum class PlyType : uint8_t { Float, Uint, Int, Uchar };

struct PlyProperty {
  std::string name;
  PlyType type;
};

struct PlyElement {
  std::string name;
  uint64_t count = 0;
  std::vector<PlyProperty> properties;
  // A property of a type this reader does not size (a list, a double...): the
  // element's rows, and those of every element after it, cannot be located.
  bool opaque = false;
  uint64_t row_bytes() const;
  // The index of a property by name, or -1.
  int find(const std::string& name) const;
};

struct PlyHeader {
  std::vector<PlyElement> elements;
  std::vector<std::string> comments;
  uint64_t body = 0;  // byte offset of the first element's first row
};

// Parses the header of a binary little-endian .ply. The vertex element must hold
// float properties only (as the reference requires); other elements may hold the
// types above, or others, which make them opaque. Errors are the reference's
// messages where it has one.
dg_status ply_parse_header(const uint8_t* bytes, uint64_t size, PlyHeader* out);

// "ply", the format line, the comments, each element and its properties, "end_header".
std::string ply_header_text(const std::vector<PlyElement>& elements, const std::vector<std::string>& comments);

// The 3DGS vertex properties in writeGaussianPly's order (src/plyWriter.ts:8-12):
// x y z nx ny nz f_dc_0..2 f_rest_0..44 opacity scale_0..2 rot_0..3.
std::vector<PlyProperty> gaussian_vertex_properties();

// One row of writeGaussianPly's body (62 floats) from a Gaussian's raw
// parameters (16 floats) and SH (45 floats, coefficient-major).
void gaussian_row(const float* params, const float* sh, float* row);

}  // namespace dg
