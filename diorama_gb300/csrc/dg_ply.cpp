// The 3D Gaussian Splatting .ply reader and writer (src/plyLoader.ts:21-104,
// src/plyWriter.ts:14-43) on the host. The reader's activation is float64
// arithmetic rounded to float32, as the reference's Float32Array stores round it.
#include "dg_ply.h"

#include <cmath>
#include <cstring>
#include <sstream>

namespace dg {

static_assert(sizeof(float) == 4, "32-bit floats");

static bool host_is_little_endian() {
  const uint32_t one = 1;
  uint8_t first;
  std::memcpy(&first, &one, 1);
  return first == 1;
}

static uint32_t type_bytes(PlyType t) { return t == PlyType::Uchar ? 1u : 4u; }

uint64_t PlyElement::row_bytes() const {
  uint64_t b = 0;
  for (const auto& p : properties) b += type_bytes(p.type);
  return b;
}

int PlyElement::find(const std::string& name) const {
  for (size_t k = 0; k < properties.size(); k++)
    if (properties[k].name == name) return (int)k;
  return -1;
}

static const char* type_name(PlyType t) {
  switch (t) {
    case PlyType::Float: return "float";
    case PlyType::Uint: return "uint";
    case PlyType::Int: return "int";
    default: return "uchar";
  }
}

static bool parse_type(const std::string& word, PlyType* out) {
  if (word == "float" || word == "float32") *out = PlyType::Float;
  else if (word == "uint" || word == "uint32") *out = PlyType::Uint;
  else if (word == "int" || word == "int32") *out = PlyType::Int;
  else if (word == "uchar" || word == "uint8") *out = PlyType::Uchar;
  else return false;
  return true;
}

static std::vector<std::string> words_of(const std::string& line) {
  std::vector<std::string> out;
  std::istringstream in(line);
  std::string w;
  while (in >> w) out.push_back(w);
  return out;
}

dg_status ply_parse_header(const uint8_t* bytes, uint64_t size, PlyHeader* out) {
  // src/plyLoader.ts:22-29: "end_header\n" within the first 64 KiB.
  static const char marker[] = "end_header\n";
  const uint64_t marker_len = sizeof(marker) - 1;
  const uint64_t limit = size < 64 * 1024 ? size : 64 * 1024;
  int64_t at = -1;
  for (uint64_t i = 0; i + marker_len <= limit; i++) {
    if (std::memcmp(bytes + i, marker, marker_len) == 0) {
      at = (int64_t)i;
      break;
    }
  }
  if (at < 0) return fail(DG_ERROR_INVALID_ARGUMENT, "No .ply header found.");
  const uint64_t header_end = (uint64_t)at + marker_len;
  const std::string header(reinterpret_cast<const char*>(bytes), header_end);
  if (header.compare(0, 4, "ply\n") != 0) return fail(DG_ERROR_INVALID_ARGUMENT, "Not a .ply file.");
  bool binary_le = false;
  std::vector<std::string> lines;
  {
    std::istringstream in(header);
    std::string line;
    while (std::getline(in, line)) {
      lines.push_back(line);
      if (line == "format binary_little_endian 1.0") binary_le = true;
    }
  }
  if (!binary_le) return fail(DG_ERROR_INVALID_ARGUMENT, "Only binary little-endian .ply files are supported.");
  if (!host_is_little_endian()) return fail(DG_ERROR_INVALID_ARGUMENT, "this host is not little-endian");
  PlyHeader h;
  for (const auto& line : lines) {
    const auto w = words_of(line);
    if (w.empty()) continue;
    if (w[0] == "comment") {
      h.comments.push_back(line.size() > 8 ? line.substr(8) : std::string());
    } else if (w[0] == "element") {
      if (w.size() < 3) return fail(DG_ERROR_INVALID_ARGUMENT, "A .ply element line needs a name and a count.");
      PlyElement e;
      e.name = w[1];
      char* end = nullptr;
      const unsigned long long n = std::strtoull(w[2].c_str(), &end, 10);
      if (end == w[2].c_str() || *end != '\0' || n > 0xffffffffull)
        return fail(DG_ERROR_INVALID_ARGUMENT, "Bad element count in the .ply header: " + w[2]);
      e.count = n;
      h.elements.push_back(e);
    } else if (w[0] == "property") {
      if (h.elements.empty() || w.size() < 3) continue;  // src/plyLoader.ts:41 skips these too
      PlyType type;
      // src/plyLoader.ts:42: vertex properties must be floats.
      if (h.elements.back().name == "vertex" && w[1] != "float")
        return fail(DG_ERROR_INVALID_ARGUMENT,
                    "Property " + w[2] + " is " + w[1] + "; only float properties are supported.");
      if (!parse_type(w[1], &type)) {
        h.elements.back().opaque = true;
        continue;
      }
      h.elements.back().properties.push_back(PlyProperty{w[2], type});
    }
  }
  if (h.elements.empty() || h.elements[0].name != "vertex")
    return fail(DG_ERROR_INVALID_ARGUMENT, "Expected the .ply to start with its vertex element.");
  h.body = header_end;
  *out = std::move(h);
  return DG_OK;
}

std::string ply_header_text(const std::vector<PlyElement>& elements, const std::vector<std::string>& comments) {
  std::string s = "ply\nformat binary_little_endian 1.0\n";
  for (const auto& c : comments) s += "comment " + c + "\n";
  for (const auto& e : elements) {
    s += "element " + e.name + " " + std::to_string(e.count) + "\n";
    for (const auto& p : e.properties) s += std::string("property ") + type_name(p.type) + " " + p.name + "\n";
  }
  s += "end_header\n";
  return s;
}

std::vector<PlyProperty> gaussian_vertex_properties() {
  std::vector<PlyProperty> p;
  for (const char* n : {"x", "y", "z", "nx", "ny", "nz", "f_dc_0", "f_dc_1", "f_dc_2"})
    p.push_back(PlyProperty{n, PlyType::Float});
  for (uint32_t k = 0; k < SH_REST_FLOATS; k++) p.push_back(PlyProperty{"f_rest_" + std::to_string(k), PlyType::Float});
  for (const char* n : {"opacity", "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3"})
    p.push_back(PlyProperty{n, PlyType::Float});
  return p;
}

// src/plyWriter.ts:28-40
void gaussian_row(const float* params, const float* sh, float* row) {
  constexpr uint32_t per_channel = SH_REST_FLOATS / 3;
  for (int k = 0; k < 3; k++) {
    row[k] = params[k];
    row[3 + k] = 0.0f;  // the normals
    row[6 + k] = params[12 + k];
  }
  // The file stores the coefficients channel by channel; training keeps them
  // coefficient by coefficient.
  for (uint32_t channel = 0; channel < 3; channel++)
    for (uint32_t c = 0; c < per_channel; c++) row[9 + channel * per_channel + c] = sh[c * 3 + channel];
  row[9 + SH_REST_FLOATS] = params[3];
  for (int k = 0; k < 3; k++) row[10 + SH_REST_FLOATS + k] = params[4 + k];
  for (int k = 0; k < 4; k++) row[13 + SH_REST_FLOATS + k] = params[8 + k];
}

}  // namespace dg

using namespace dg;

dg_status dg_parse_gaussian_ply(const void* data, uint64_t size, uint32_t* count, uint32_t* sh_degree,
                                float* gaussians, float* sh_rest) {
  DG_REQUIRE(data && count && sh_degree, "NULL argument");
  const uint8_t* bytes = static_cast<const uint8_t*>(data);
  PlyHeader h;
  DG_TRY(ply_parse_header(bytes, size, &h));
  const PlyElement& v = h.elements[0];
  auto column = [&](const std::string& name, int* out) -> dg_status {
    const int k = v.find(name);
    if (k < 0)
      return fail(DG_ERROR_INVALID_ARGUMENT,
                  "The .ply has no \"" + name + "\" property. Is it a 3D Gaussian Splatting file?");
    *out = k;
    return DG_OK;
  };
  int position[3], dc[3], scale[3], rotation[4], opacity;
  for (int k = 0; k < 3; k++) {
    DG_TRY(column(std::string(1, (char)('x' + k)), &position[k]));
    DG_TRY(column("f_dc_" + std::to_string(k), &dc[k]));
  }
  DG_TRY(column("opacity", &opacity));
  for (int k = 0; k < 3; k++) DG_TRY(column("scale_" + std::to_string(k), &scale[k]));
  for (int k = 0; k < 4; k++) DG_TRY(column("rot_" + std::to_string(k), &rotation[k]));
  // src/plyLoader.ts:57-62
  uint32_t rest_count = 0;
  for (const auto& p : v.properties)
    if (p.name.compare(0, 7, "f_rest_") == 0) rest_count++;
  const double per_channel_f = rest_count / 3.0;
  const int degree = (int)std::lround(std::sqrt(per_channel_f + 1.0)) - 1;
  if ((double)((degree + 1) * (degree + 1) - 1) != per_channel_f || degree > 3)
    return fail(DG_ERROR_INVALID_ARGUMENT,
                "Unexpected number of spherical-harmonic coefficients (" + std::to_string(rest_count) + ").");
  const uint32_t per_channel = rest_count / 3;
  std::vector<int> rest(rest_count);
  for (uint32_t k = 0; k < rest_count; k++) DG_TRY(column("f_rest_" + std::to_string(k), &rest[k]));
  const uint64_t stride = v.properties.size();
  if (h.body + v.count * stride * 4 > size)
    return fail(DG_ERROR_INVALID_ARGUMENT, "The .ply file is shorter than its header says.");
  *count = (uint32_t)v.count;
  *sh_degree = (uint32_t)degree;
  if (!gaussians && !sh_rest) return DG_OK;
  DG_REQUIRE(gaussians && sh_rest, "gaussians and sh_rest must both be given");
  const double sh_c0 = 0.28209479177387814;
  std::vector<float> row(stride);
  for (uint64_t i = 0; i < v.count; i++) {
    std::memcpy(row.data(), bytes + h.body + i * stride * 4, stride * 4);
    float* g = gaussians + i * FLOATS_PER_GAUSSIAN;
    // src/plyLoader.ts:83-100
    for (int k = 0; k < 3; k++) {
      g[k] = row[position[k]];
      g[4 + k] = (float)std::exp((double)row[scale[k]]);
      g[12 + k] = (float)(0.5 + sh_c0 * (double)row[dc[k]]);
    }
    g[3] = (float)(1.0 / (1.0 + std::exp(-(double)row[opacity])));
    for (int k = 0; k < 4; k++) g[8 + k] = row[rotation[k]];
    g[7] = g[15] = 0.0f;
    float* s = sh_rest + i * SH_REST_FLOATS;
    std::memset(s, 0, SH_REST_FLOATS * sizeof(float));
    for (uint32_t c = 0; c < per_channel; c++)
      for (uint32_t channel = 0; channel < 3; channel++) s[c * 3 + channel] = row[rest[channel * per_channel + c]];
  }
  return DG_OK;
}

dg_status dg_write_gaussian_ply(const float* params, const float* sh, uint32_t count, void* out, uint64_t capacity,
                                uint64_t* size) {
  DG_REQUIRE(size && (count == 0 || (params && sh)), "NULL argument");
  PlyElement vertex;
  vertex.name = "vertex";
  vertex.count = count;
  vertex.properties = gaussian_vertex_properties();
  const std::string header = ply_header_text({vertex}, {});
  const uint64_t stride = vertex.properties.size();
  *size = header.size() + (uint64_t)count * stride * 4;
  if (!out) return DG_OK;
  DG_REQUIRE(capacity >= *size, "output buffer too small");
  uint8_t* o = static_cast<uint8_t*>(out);
  std::memcpy(o, header.data(), header.size());
  std::vector<float> row(stride);
  for (uint32_t i = 0; i < count; i++) {
    gaussian_row(params + (size_t)i * FLOATS_PER_GAUSSIAN, sh + (size_t)i * SH_REST_FLOATS, row.data());
    std::memcpy(o + header.size() + (uint64_t)i * stride * 4, row.data(), stride * 4);
  }
  return DG_OK;
}
