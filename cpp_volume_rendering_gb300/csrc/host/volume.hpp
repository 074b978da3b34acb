// volume.hpp — host mirror of vis::StructuredGridVolume and its readers
// (libs/volvis_utils/structuredgridvolume.h:40-88, reader.cpp:28-628,
// libs/file_utils/rawloader.cpp:5-42).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace vis {

enum class DataStorageSize { UNKNOWN = 0, _8_BITS = 1, _16_BITS = 2 };

class StructuredGridVolume {
 public:
  StructuredGridVolume() = default;
  StructuredGridVolume(const std::string& name, int w, int h, int d);

  int GetWidth() const { return m_w; }
  int GetHeight() const { return m_h; }
  int GetDepth() const { return m_d; }
  double GetScaleX() const { return m_sx; }
  double GetScaleY() const { return m_sy; }
  double GetScaleZ() const { return m_sz; }
  void SetScale(double x, double y, double z) { m_sx = x; m_sy = y; m_sz = z; }
  double GetDiagonal() const;                 // structuredgridvolume.cpp:96-102
  DataStorageSize GetStorage() const { return m_storage; }
  size_t GetBytesPerVoxel() const { return m_storage == DataStorageSize::_16_BITS ? 2 : 1; }
  size_t GetNumVoxels() const { return (size_t)m_w * m_h * m_d; }

  // Takes ownership of a copy of the voxels.
  void SetArrayData(const void* data, DataStorageSize dss);
  const void* GetArrayData() const { return m_bytes.empty() ? nullptr : m_bytes.data(); }
  void* GetArrayDataMutable() { return m_bytes.empty() ? nullptr : m_bytes.data(); }
  // structuredgridvolume.cpp:121-151: v / 255 or v / 65535, 0 outside.
  double GetNormalizedSample(int x, int y, int z) const;

  std::string name;

 private:
  int m_w = 0, m_h = 0, m_d = 0;
  double m_sx = 1.0, m_sy = 1.0, m_sz = 1.0;
  DataStorageSize m_storage = DataStorageSize::UNKNOWN;
  std::vector<uint8_t> m_bytes;
};

// Parses the readraw file name convention "<name>.<bytes>.<W>x<H>x<D>.raw"
// (reader.cpp:162-225).  Returns false on a malformed name.
bool ParseRawName(const std::string& path, int* w, int* h, int* d, int* bytes_per_value);

// VolumeReader::ReadStructuredVolume dispatch on the extension (.raw, .syn,
// .pvm / .pvmold, .nrrd / .nhrd, .dat).  Returns false (with a message)
// instead of exiting on a missing, short or malformed file.
bool ReadStructuredVolume(const std::string& path, StructuredGridVolume* out, std::string* err);
// The readers of readers.cpp (also reached through ReadStructuredVolume).
bool ReadPVM(const std::string& path, StructuredGridVolume* out, std::string* err);
bool ReadNRRD(const std::string& path, StructuredGridVolume* out, std::string* err);
bool ReadDAT(const std::string& path, StructuredGridVolume* out, std::string* err);

// Camera / light list files (camerastatelist.cpp:26-87, lightsourcelist.cpp:81-148).
struct CameraState {
  std::string name;
  int type = 0;  // 0 ARCBALL, 1 FLIGHT
  float eye[3] = {0, 0, 0}, center[3] = {0, 0, 0}, up[3] = {0, 0, 0};
};
bool ReadCameraStates(const std::string& path, std::vector<CameraState>* out, std::string* err);

struct LightSourceData {
  float position[3] = {0, 0, 0};
  float z_axis[3] = {0, 0, 1};  // = -forward as read from the file
  float y_axis[3] = {0, 1, 0};
  float x_axis[3] = {1, 0, 0};
  float spot_light_angle = 4.0f;
  float specular[3] = {1, 1, 1};  // LightSourceData::specular (lightsourcelist.cpp:24)
};
struct LightSourceList {
  std::string name;
  std::vector<LightSourceData> lights;
};
bool ReadLightSourceLists(const std::string& path, std::vector<LightSourceList>* out, std::string* err);

}  // namespace vis
