// A COLMAP sparse reconstruction (cameras.bin, images.bin, points3D.bin) on the
// host (src/colmap.ts:18-129): each registered photo's camera, sorted by file
// name, and the structure-from-motion points. The pose arithmetic is float64, as
// the reference's numbers are; the points are rounded to float32 as its
// Float32Array stores round them.
#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "dg_common.cuh"

struct dg_colmap {
  std::vector<dg_training_camera> cameras;
  std::vector<std::string> names;  // cameras[k].name points into names[k]
  std::vector<float> positions;
  std::vector<uint8_t> colors;
};

namespace dg {
namespace {

// Little-endian reads over one file's bytes (src/colmap.ts:33-67). Reading past
// the end fails instead of throwing a RangeError as a DataView does.
struct Reader {
  const uint8_t* data;
  uint64_t size, offset = 0;
  const char* file;
  bool ok = true;

  bool take(void* out, uint64_t bytes) {
    if (!ok || bytes > size - offset) {
      ok = false;
      std::memset(out, 0, bytes);
      return false;
    }
    std::memcpy(out, data + offset, bytes);
    offset += bytes;
    return true;
  }
  uint8_t u8() {
    uint8_t v;
    take(&v, 1);
    return v;
  }
  int32_t i32() {
    uint8_t b[4];
    take(b, 4);
    return (int32_t)((uint32_t)b[0] | (uint32_t)b[1] << 8 | (uint32_t)b[2] << 16 | (uint32_t)b[3] << 24);
  }
  uint64_t u64() {
    uint8_t b[8];
    take(b, 8);
    uint64_t v = 0;
    for (int k = 7; k >= 0; k--) v = v << 8 | b[k];
    return v;
  }
  double f64() {
    const uint64_t bits = u64();
    double v;
    std::memcpy(&v, &bits, 8);
    return v;
  }
  void skip(uint64_t bytes) {
    if (!ok || bytes > size - offset) ok = false;
    else offset += bytes;
  }
  std::string string() {
    const uint64_t start = offset;
    while (ok && offset < size && data[offset] != 0) offset++;
    if (offset >= size) {
      ok = false;
      return std::string();
    }
    std::string s(reinterpret_cast<const char*>(data + start), offset - start);
    offset++;  // the terminating zero
    return s;
  }
};

struct Intrinsics {
  double width, height, fx, fy;
};

dg_status truncated(const Reader& r) {
  return fail(DG_ERROR_INVALID_ARGUMENT, std::string(r.file) + " is shorter than its contents say.");
}

// src/colmap.ts:71-94
dg_status read_cameras(Reader& r, std::map<int32_t, Intrinsics>* out) {
  for (uint64_t count = r.u64(); count > 0 && r.ok; count--) {
    const int32_t id = r.i32();
    const int32_t model = r.i32();
    const double width = (double)r.u64(), height = (double)r.u64();
    if (!r.ok) break;
    if (model == 0) {  // SIMPLE_PINHOLE: f, cx, cy
      const double f = r.f64();
      r.skip(16);
      (*out)[id] = Intrinsics{width, height, f, f};
    } else if (model == 1) {  // PINHOLE: fx, fy, cx, cy
      const double fx = r.f64(), fy = r.f64();
      r.skip(16);
      (*out)[id] = Intrinsics{width, height, fx, fy};
    } else {
      return fail(DG_ERROR_INVALID_ARGUMENT, "Camera " + std::to_string(id) + " uses COLMAP model " +
                                                 std::to_string(model) +
                                                 "; only undistorted pinhole cameras are supported.");
    }
  }
  return r.ok ? DG_OK : truncated(r);
}

// src/colmap.ts:121-128: the rotation of a unit quaternion (w, x, y, z).
void rotation_matrix(const double q[4], double m[3][3]) {
  const double w = q[0], x = q[1], y = q[2], z = q[3];
  m[0][0] = 1 - 2 * (y * y + z * z);
  m[0][1] = 2 * (x * y - w * z);
  m[0][2] = 2 * (x * z + w * y);
  m[1][0] = 2 * (x * y + w * z);
  m[1][1] = 1 - 2 * (x * x + z * z);
  m[1][2] = 2 * (y * z - w * x);
  m[2][0] = 2 * (x * z - w * y);
  m[2][1] = 2 * (y * z + w * x);
  m[2][2] = 1 - 2 * (x * x + y * y);
}

}  // namespace
}  // namespace dg

using namespace dg;

dg_status dg_parse_colmap(const void* cameras_bin, uint64_t cameras_size, const void* images_bin,
                          uint64_t images_size, const void* points_bin, uint64_t points_size, dg_colmap** out) {
  DG_REQUIRE(out && (cameras_bin || !cameras_size) && (images_bin || !images_size) && (points_bin || !points_size),
             "NULL argument");
  std::map<int32_t, Intrinsics> intrinsics;
  Reader cams{static_cast<const uint8_t*>(cameras_bin), cameras_size, 0, "cameras.bin"};
  DG_TRY(read_cameras(cams, &intrinsics));
  auto* rec = new dg_colmap();
  auto bail = [&](dg_status st) {
    delete rec;
    return st;
  };
  // src/colmap.ts:96-108 and 19-30
  Reader images{static_cast<const uint8_t*>(images_bin), images_size, 0, "images.bin"};
  struct Photo {
    std::string name;
    dg_training_camera camera;
  };
  std::vector<Photo> photos;
  for (uint64_t count = images.u64(); count > 0 && images.ok; count--) {
    images.i32();  // image id
    double q[4], t[3];
    for (double& v : q) v = images.f64();
    for (double& v : t) v = images.f64();
    const int32_t camera_id = images.i32();
    std::string name = images.string();
    images.skip(images.u64() * 24);  // the photo's 2D points: x, y and a point id each
    if (!images.ok) break;
    const auto it = intrinsics.find(camera_id);
    if (it == intrinsics.end())
      return bail(fail(DG_ERROR_INVALID_ARGUMENT, "Photo " + name + " uses camera " + std::to_string(camera_id) +
                                                      ", which isn't in cameras.bin."));
    // COLMAP stores world -> camera: x_camera = R x_world + t. The camera sits at
    // -R^T t, and R's rows are its axes in world space (x right, y down, z forward).
    double r[3][3];
    rotation_matrix(q, r);
    dg_training_camera c{};
    c.width = it->second.width;
    c.height = it->second.height;
    c.fx = it->second.fx;
    c.fy = it->second.fy;
    for (int k = 0; k < 3; k++) {
      c.position[k] = -(r[0][k] * t[0] + r[1][k] * t[1] + r[2][k] * t[2]);
      c.right[k] = r[0][k];
      c.down[k] = r[1][k];
      c.forward[k] = r[2][k];
    }
    photos.push_back(Photo{std::move(name), c});
  }
  if (!images.ok) return bail(truncated(images));
  // Sorted by file name, as a JavaScript string comparison orders them (by UTF-16
  // code units; byte order agrees with it for names without characters beyond
  // U+FFFF).
  std::stable_sort(photos.begin(), photos.end(), [](const Photo& a, const Photo& b) { return a.name < b.name; });
  // src/colmap.ts:110-119
  Reader points{static_cast<const uint8_t*>(points_bin), points_size, 0, "points3D.bin"};
  const uint64_t count = points.u64();
  if (!points.ok || count > (points_size - 8) / 51) return bail(truncated(points));  // 51: a record's least size
  rec->positions.resize(count * 3);
  rec->colors.resize(count * 3);
  for (uint64_t i = 0; i < count && points.ok; i++) {
    points.u64();  // point id
    for (int k = 0; k < 3; k++) rec->positions[i * 3 + k] = (float)points.f64();
    for (int k = 0; k < 3; k++) rec->colors[i * 3 + k] = points.u8();
    points.f64();                      // reprojection error
    points.skip(points.u64() * 8);     // which photos saw it: an image id and point index each
  }
  if (!points.ok) return bail(truncated(points));
  rec->names.reserve(photos.size());
  for (auto& p : photos) rec->names.push_back(std::move(p.name));
  for (size_t k = 0; k < photos.size(); k++) {
    rec->cameras.push_back(photos[k].camera);
    rec->cameras.back().name = rec->names[k].c_str();
  }
  *out = rec;
  return DG_OK;
}

uint32_t dg_colmap_camera_count(const dg_colmap* r) { return r ? (uint32_t)r->cameras.size() : 0; }

dg_status dg_colmap_camera(const dg_colmap* r, uint32_t index, dg_training_camera* out) {
  DG_REQUIRE(r && out, "NULL argument");
  DG_REQUIRE(index < r->cameras.size(), "camera index out of range");
  *out = r->cameras[index];
  return DG_OK;
}

uint64_t dg_colmap_point_count(const dg_colmap* r) { return r ? r->colors.size() / 3 : 0; }

dg_status dg_colmap_points(const dg_colmap* r, float* positions, uint8_t* colors) {
  DG_REQUIRE(r && (r->colors.empty() || (positions && colors)), "NULL argument");
  if (!r->positions.empty()) std::memcpy(positions, r->positions.data(), r->positions.size() * 4);
  if (!r->colors.empty()) std::memcpy(colors, r->colors.data(), r->colors.size());
  return DG_OK;
}

dg_status dg_colmap_destroy(dg_colmap* r) {
  delete r;
  return DG_OK;
}
