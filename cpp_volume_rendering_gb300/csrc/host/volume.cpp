// volume.cpp — StructuredGridVolume and the .raw / .syn / list readers.
// Portable restatement: the reference's MSVC-only fopen_s and unsigned char(v)
// casts (rawloader.cpp:14-16, reader.cpp:317,352) become plain C++.
#include "volume.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>

namespace vis {

StructuredGridVolume::StructuredGridVolume(const std::string& n, int w, int h, int d)
    : name(n), m_w(w), m_h(h), m_d(d) {}

double StructuredGridVolume::GetDiagonal() const {
  double vw = m_w * m_sx, vh = m_h * m_sy, vd = m_d * m_sz;
  return std::sqrt(vw * vw + vh * vh + vd * vd);
}

void StructuredGridVolume::SetArrayData(const void* data, DataStorageSize dss) {
  m_storage = dss;
  size_t n = GetNumVoxels() * (dss == DataStorageSize::_16_BITS ? 2 : 1);
  m_bytes.resize(n);
  if (data && n) std::memcpy(m_bytes.data(), data, n);
}

double StructuredGridVolume::GetNormalizedSample(int x, int y, int z) const {
  if (m_bytes.empty() || m_storage == DataStorageSize::UNKNOWN || x < 0 || y < 0 || z < 0 || x >= m_w ||
      y >= m_h || z >= m_d)
    return 0.0;
  size_t i = (size_t)x + (size_t)y * m_w + (size_t)z * m_w * m_h;
  if (m_storage == DataStorageSize::_8_BITS) return (double)m_bytes[i] / (256.0 - 1.0);
  uint16_t v;
  std::memcpy(&v, m_bytes.data() + 2 * i, 2);
  return (double)v / (65536.0 - 1.0);
}

bool ParseRawName(const std::string& path, int* w, int* h, int* d, int* bytes_per_value) {
  // strip directories (both separators) and the extension
  size_t slash = path.find_last_of("/\\");
  std::string name = slash == std::string::npos ? path : path.substr(slash + 1);
  size_t dot = name.find_last_of('.');
  if (dot == std::string::npos) return false;
  name = name.substr(0, dot);
  size_t ds = name.find_last_of('.');
  if (ds == std::string::npos) return false;
  std::string sizes = name.substr(ds + 1);
  name = name.substr(0, ds);
  size_t db = name.find_last_of('.');
  if (db == std::string::npos) return false;
  std::string bytes = name.substr(db + 1);
  int vals[3];
  for (int k = 2; k >= 0; --k) {
    size_t x = sizes.find_last_of('x');
    std::string tok = (k == 0) ? sizes : (x == std::string::npos ? std::string() : sizes.substr(x + 1));
    if (tok.empty()) return false;
    char* end = nullptr;
    long v = std::strtol(tok.c_str(), &end, 10);
    if (*end != '\0' || v <= 0 || v > (1 << 16)) return false;
    vals[k] = (int)v;
    if (k > 0) sizes = sizes.substr(0, x);
  }
  char* end = nullptr;
  long b = std::strtol(bytes.c_str(), &end, 10);
  if (*end != '\0' || (b != 1 && b != 2)) return false;
  *w = vals[0]; *h = vals[1]; *d = vals[2]; *bytes_per_value = (int)b;
  return true;
}

static bool read_raw(const std::string& path, StructuredGridVolume* out, std::string* err) {
  int w, h, d, bpv;
  if (!ParseRawName(path, &w, &h, &d, &bpv)) {
    if (err) *err = "raw file name must be <name>.<bytes>.<W>x<H>x<D>.raw: " + path;
    return false;
  }
  FILE* fp = std::fopen(path.c_str(), "rb");
  if (!fp) {
    if (err) *err = "opening .raw file failed: " + path;
    return false;
  }
  size_t n = (size_t)w * h * d;
  std::vector<uint8_t> buf(n * bpv);
  size_t got = std::fread(buf.data(), (size_t)bpv, n, fp);
  std::fclose(fp);
  if (got != n) {
    if (err) *err = "short .raw file: " + std::to_string(got) + " values read, " + std::to_string(n) + " expected";
    return false;
  }
  *out = StructuredGridVolume(path, w, h, d);
  out->SetScale(1.0, 1.0, 1.0);
  out->SetArrayData(buf.data(), bpv == 2 ? DataStorageSize::_16_BITS : DataStorageSize::_8_BITS);
  return true;
}

// readsyn (reader.cpp:283-371): "W H D" then records "1 x0 y0 z0 x1 y1 z1 v"
// (box fill) or "<other> x y z v" (single voxel); u8 voxels.  Voxels no record
// touches are zero here (the reference leaves them uninitialised).
static bool read_syn(const std::string& path, StructuredGridVolume* out, std::string* err) {
  std::ifstream f(path);
  if (!f.is_open()) {
    if (err) *err = "opening .syn file failed: " + path;
    return false;
  }
  int w, h, d;
  if (!(f >> w >> h >> d) || w <= 0 || h <= 0 || d <= 0 || (double)w * h * d > 4.0e9) {
    if (err) *err = "malformed .syn header: " + path;
    return false;
  }
  std::vector<uint8_t> data((size_t)w * h * d, 0);
  int kind;
  while (f >> kind) {
    if (kind == 1) {
      int x0, y0, z0, x1, y1, z1, v;
      if (!(f >> x0 >> y0 >> z0 >> x1 >> y1 >> z1 >> v)) {
        if (err) *err = "truncated .syn box record: " + path;
        return false;
      }
      for (int x = std::max(x0, 0); x < std::min(x1, w); ++x)
        for (int y = std::max(y0, 0); y < std::min(y1, h); ++y)
          for (int z = std::max(z0, 0); z < std::min(z1, d); ++z)
            data[(size_t)x + (size_t)w * y + (size_t)w * h * z] = (uint8_t)v;
    } else {
      int x, y, z, v;
      if (!(f >> x >> y >> z >> v)) {
        if (err) *err = "truncated .syn voxel record: " + path;
        return false;
      }
      if (x >= 0 && y >= 0 && z >= 0 && x < w && y < h && z < d)
        data[(size_t)x + (size_t)w * y + (size_t)w * h * z] = (uint8_t)v;
    }
  }
  *out = StructuredGridVolume(path, w, h, d);
  out->SetScale(1.0, 1.0, 1.0);
  out->SetArrayData(data.data(), DataStorageSize::_8_BITS);
  return true;
}

bool ReadStructuredVolume(const std::string& path, StructuredGridVolume* out, std::string* err) {
  size_t dot = path.find_last_of('.');
  std::string ext = dot == std::string::npos ? std::string() : path.substr(dot + 1);
  if (ext == "raw") return read_raw(path, out, err);
  if (ext == "syn") return read_syn(path, out, err);
  if (ext == "pvm" || ext == "pvmold") return ReadPVM(path, out, err);  // one format, two reference loaders
  if (ext == "nrrd" || ext == "nhrd") return ReadNRRD(path, out, err);
  if (ext == "dat") return ReadDAT(path, out, err);
  if (err) *err = "unsupported volume format: ." + ext;
  return false;
}

static void trim_cr(std::string& s) {
  while (!s.empty() && (s.back() == '\r' || s.back() == '\n')) s.pop_back();
}

bool ReadCameraStates(const std::string& path, std::vector<CameraState>* out, std::string* err) {
  out->clear();
  std::ifstream f(path);
  if (!f.is_open()) {
    if (err) *err = "Unable to read camera states: " + path;
    return false;
  }
  std::string line;
  while (std::getline(f, line)) {
    trim_cr(line);
    if (line.empty() && f.eof()) break;
    CameraState c;
    c.name = line;
    std::string kind;
    if (!std::getline(f, kind)) break;
    trim_cr(kind);
    if (kind == "FLIGHT") {
      c.type = 1;
    } else if (kind == "ARCBALL") {
      c.type = 0;
      if (!(f >> c.eye[0] >> c.eye[1] >> c.eye[2] >> c.center[0] >> c.center[1] >> c.center[2] >> c.up[0] >>
            c.up[1] >> c.up[2])) {
        if (err) *err = "truncated camera state '" + c.name + "'";
        return false;
      }
      std::getline(f, line);
    }
    out->push_back(c);
  }
  return !out->empty();
}

bool ReadLightSourceLists(const std::string& path, std::vector<LightSourceList>* out, std::string* err) {
  out->clear();
  std::ifstream f(path);
  if (!f.is_open()) {
    if (err) *err = "Unable to read light source list: " + path;
    return false;
  }
  std::string line;
  while (std::getline(f, line)) {
    trim_cr(line);
    if (line.empty() && f.eof()) break;
    LightSourceList l;
    l.name = line;
    int n = 0;
    if (!(f >> n) || n < 0 || n > 4096) {
      if (err) *err = "malformed light count in list '" + l.name + "'";
      return false;
    }
    for (int i = 0; i < n; ++i) {
      LightSourceData ld;
      float fwd[3];
      if (!(f >> ld.position[0] >> ld.position[1] >> ld.position[2] >> fwd[0] >> fwd[1] >> fwd[2] >> ld.y_axis[0] >>
            ld.y_axis[1] >> ld.y_axis[2] >> ld.x_axis[0] >> ld.x_axis[1] >> ld.x_axis[2] >> ld.spot_light_angle)) {
        if (err) *err = "truncated light in list '" + l.name + "'";
        return false;
      }
      for (int k = 0; k < 3; ++k) ld.z_axis[k] = -fwd[k];
      std::getline(f, line);
      l.lights.push_back(ld);
    }
    out->push_back(l);
  }
  return !out->empty();
}

}  // namespace vis
