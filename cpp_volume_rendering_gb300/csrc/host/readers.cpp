// readers.cpp — the .pvm (optionally DDS-compressed), .nrrd / .nhrd and .dat
// volume readers of VolumeReader::ReadStructuredVolume
// (libs/volvis_utils/reader.cpp:28-58), written from the published formats:
//
//  * PVM (V^3 volume format): "PVM\n" [# comment lines] "W H D\n" "C\n" data,
//    or "PVM2\n"/"PVM3\n" "W H D\n" "sx sy sz\n" "C\n" data [PVM3: four
//    NUL-terminated strings after it]; C bytes per voxel.
//  * DDS (differential data stream) around it: "DDS v3d\n" (no blocking) or
//    "DDS v3e\n" (interleave blocks of 2^24), then an MSB-first bit stream:
//    skip-1 (2 bits), strip-1 (16 bits), then runs "count (7 bits, 0 ends)
//    code (3 bits; bits = code + 1 for code >= 1)" of count residuals of
//    'bits' bits, each value = previous value (+ the value strip bytes back
//    minus its predecessor, past the first strip bytes) + residual - 2^bits/2,
//    mod 256; the byte stream was deinterleaved by 'skip' (all bytes of
//    phase 0, then phase 1, ...) within each block.
//  * NRRD: "key: value" header lines; the reference reads "sizes", "type"
//    (uint8 / uint16) and a detached "data file" of raw voxels, spacing 1
//    (reader.cpp:373-491).
//  * .dat: "ObjectFileName", "Resolution", "SliceThickness", "Format"
//    (UCHAR / USHORT) lines and a raw file next to it (reader.cpp:498-628).
//
// Where the reference exits the process on a malformed file these return
// false with a message.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "volume.hpp"

namespace vis {
namespace {

bool fail(std::string* err, const std::string& msg) {
  if (err) *err = msg;
  return false;
}

bool slurp(const std::string& path, std::vector<uint8_t>* out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  out->clear();
  uint8_t buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) out->insert(out->end(), buf, buf + n);
  std::fclose(f);
  return true;
}

// MSB-first bit reader (at most 24 bits per read); bits past the end read as zeros.
class BitStream {
 public:
  BitStream(const uint8_t* p, size_t n) : m_p(p), m_n(n) {}
  uint32_t Read(int bits) {
    if (bits == 0) return 0;
    while (m_have < bits) {  // append the next byte below the buffered bits
      m_buf = (m_buf << 8) | (m_next < m_n ? m_p[m_next] : 0u);
      ++m_next;
      m_have += 8;
    }
    m_have -= bits;
    return (uint32_t)(m_buf >> m_have) & ((1u << bits) - 1u);
  }

 private:
  const uint8_t* m_p;
  size_t m_n;
  size_t m_next = 0;  // next byte to append
  uint64_t m_buf = 0;
  int m_have = 0;     // valid bits at the bottom of m_buf
};

// Puts a deinterleaved byte stream back in order: within each block of
// skip*block bytes (block 0: the whole stream) the bytes were stored phase
// by phase (positions i, i+skip, i+2 skip, ... for i = 0 .. skip-1).
void restore_interleave(std::vector<uint8_t>& d, unsigned skip, size_t block) {
  if (skip <= 1 || d.empty()) return;
  const size_t chunk = block == 0 ? d.size() : (size_t)skip * block;
  std::vector<uint8_t> tmp(std::min(chunk, d.size()));
  for (size_t base = 0; base < d.size(); base += chunk) {
    const size_t len = std::min(chunk, d.size() - base);
    size_t src = base;
    for (unsigned i = 0; i < skip; ++i)
      for (size_t j = i; j < len; j += skip) tmp[j] = d[src++];
    std::memcpy(d.data() + base, tmp.data(), len);
  }
}

bool dds_unpack(const uint8_t* p, size_t n, size_t block, std::vector<uint8_t>* out, std::string* err) {
  BitStream bs(p, n);
  const unsigned skip = bs.Read(2) + 1;
  const size_t strip = (size_t)bs.Read(16) + 1;
  out->clear();
  int act = 0;
  for (;;) {
    const uint32_t count = bs.Read(7);
    if (count == 0) break;
    const uint32_t code = bs.Read(3);
    const int bits = code >= 1 ? (int)code + 1 : 0;
    const int half = (1 << bits) / 2;
    for (uint32_t k = 0; k < count; ++k) {
      const size_t cnt = out->size();
      int pred = act;
      if (strip > 1 && cnt > strip) pred += (int)(*out)[cnt - strip] - (int)(*out)[cnt - strip - 1];
      act = (pred + (int)bs.Read(bits) - half) & 255;
      out->push_back((uint8_t)act);
    }
    if (out->size() > ((size_t)1 << 36)) return fail(err, "DDS stream decodes to more than 64 GiB");
  }
  restore_interleave(*out, skip, block);
  return true;
}

// Next line of a text header starting at *pos (without the '\n'); false at the end.
bool next_line(const std::vector<uint8_t>& b, size_t* pos, std::string* line) {
  if (*pos >= b.size()) return false;
  const uint8_t* s = b.data() + *pos;
  const void* nl = std::memchr(s, '\n', b.size() - *pos);
  const size_t len = nl ? (size_t)((const uint8_t*)nl - s) : b.size() - *pos;
  line->assign((const char*)s, len);
  *pos += len + (nl ? 1 : 0);
  return true;
}

// readpvm (reader.cpp:100-160) over DDSV3::readPVMvolume's format; 16-bit
// voxels are assembled as byte0 + 256 * byte1 (Pvm::PostProcessData).
bool read_pvm(const std::string& path, StructuredGridVolume* out, std::string* err) {
  std::vector<uint8_t> file;
  if (!slurp(path, &file)) return fail(err, "opening .pvm file failed: " + path);
  std::vector<uint8_t> plain;
  const std::vector<uint8_t>* b = &file;
  if (file.size() >= 8 && (std::memcmp(file.data(), "DDS v3d\n", 8) == 0 || std::memcmp(file.data(), "DDS v3e\n", 8) == 0)) {
    const size_t block = file[6] == 'd' ? 0 : ((size_t)1 << 24);
    if (!dds_unpack(file.data() + 8, file.size() - 8, block, &plain, err)) return false;
    b = &plain;
  }
  size_t pos = 0;
  std::string line;
  if (!next_line(*b, &pos, &line)) return fail(err, "empty .pvm file: " + path);
  int version;
  if (line == "PVM") version = 1;
  else if (line == "PVM2") version = 2;
  else if (line == "PVM3") version = 3;
  else return fail(err, "not a PVM volume (magic '" + line.substr(0, 8) + "'): " + path);
  long w = 0, h = 0, d = 0, c = 0;
  double sx = 1.0, sy = 1.0, sz = 1.0;
  do {
    if (!next_line(*b, &pos, &line)) return fail(err, "truncated .pvm header: " + path);
  } while (version == 1 && !line.empty() && line[0] == '#');
  if (std::sscanf(line.c_str(), "%ld %ld %ld", &w, &h, &d) != 3 || w < 1 || h < 1 || d < 1)
    return fail(err, "malformed .pvm dimensions '" + line + "': " + path);
  if (version > 1) {
    float fx, fy, fz;
    if (!next_line(*b, &pos, &line) || std::sscanf(line.c_str(), "%g %g %g", &fx, &fy, &fz) != 3 ||
        !(fx > 0.0f && fy > 0.0f && fz > 0.0f))
      return fail(err, "malformed .pvm voxel spacing: " + path);
    sx = fx; sy = fy; sz = fz;
  }
  if (!next_line(*b, &pos, &line) || std::sscanf(line.c_str(), "%ld", &c) != 1 || c < 1)
    return fail(err, "malformed .pvm component count: " + path);
  if (c > 2) return fail(err, ".pvm with " + std::to_string(c) + " bytes per voxel (only 1 and 2 are volumes): " + path);
  if ((double)w * h * d > 17179869184.0) return fail(err, ".pvm volume too large: " + path);
  const size_t n = (size_t)w * h * d * (size_t)c;
  if (b->size() - pos < n) return fail(err, "short .pvm data: " + path);
  if (version < 3 && b->size() - pos != n) return fail(err, ".pvm data size does not match its header: " + path);
  *out = StructuredGridVolume(path, (int)w, (int)h, (int)d);
  out->SetScale(sx, sy, sz);
  if (c == 1) {
    out->SetArrayData(b->data() + pos, DataStorageSize::_8_BITS);
  } else {
    std::vector<uint16_t> v((size_t)w * h * d);
    const uint8_t* p = b->data() + pos;
    for (size_t i = 0; i < v.size(); ++i) v[i] = (uint16_t)(p[2 * i] + 256u * p[2 * i + 1]);
    out->SetArrayData(v.data(), DataStorageSize::_16_BITS);
  }
  return true;
}

// "key: value" with the value's leading blanks and a trailing '\r' removed.
bool key_value(std::string line, std::string* key, std::string* value) {
  if (!line.empty() && line.back() == '\r') line.pop_back();
  const size_t colon = line.find(':');
  if (colon == std::string::npos) return false;
  *key = line.substr(0, colon);
  size_t s = colon + 1;
  while (s < line.size() && (line[s] == ' ' || line[s] == '\t')) ++s;
  *value = line.substr(s);
  return true;
}

std::string directory_of(const std::string& path) {
  const size_t slash = path.find_last_of("/\\");
  return slash == std::string::npos ? std::string(".") : path.substr(0, slash);
}

bool read_raw_values(const std::string& path, int w, int h, int d, int bpv, StructuredGridVolume* out,
                     std::string* err) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return fail(err, "opening raw data file failed: " + path);
  const size_t n = (size_t)w * h * d;
  std::vector<uint8_t> buf(n * (size_t)bpv);
  const size_t got = std::fread(buf.data(), (size_t)bpv, n, f);
  std::fclose(f);
  if (got != n)
    return fail(err, "short raw data file: " + std::to_string(got) + " values read, " + std::to_string(n) + " expected");
  out->SetArrayData(buf.data(), bpv == 2 ? DataStorageSize::_16_BITS : DataStorageSize::_8_BITS);
  return true;
}

bool three_ints(const std::string& s, long* v) {
  std::istringstream is(s);
  return static_cast<bool>(is >> v[0] >> v[1] >> v[2]) && v[0] > 0 && v[1] > 0 && v[2] > 0 &&
         (double)v[0] * v[1] * v[2] <= 17179869184.0;
}

// readnrrd (reader.cpp:373-491).  Keys are matched by prefix in the
// reference's order, so "space directions" / "space origin" fall under
// "space" and the spacing stays 1.
bool read_nrrd(const std::string& path, StructuredGridVolume* out, std::string* err) {
  std::ifstream f(path);
  if (!f.is_open()) return fail(err, "opening .nrrd file failed: " + path);
  std::string line, key, value, type, data_file;
  long dims[3] = {0, 0, 0};
  bool have_sizes = false;
  std::getline(f, line);  // NRRD000x magic
  if (line.compare(0, 4, "NRRD") != 0) return fail(err, "not a NRRD header: " + path);
  while (std::getline(f, line)) {
    if (!line.empty() && line[0] == '#') continue;
    if (line.empty() || line == "\r") break;  // end of the header
    if (!key_value(line, &key, &value)) continue;
    if (key.rfind("type", 0) == 0) type = value;
    else if (key.rfind("sizes", 0) == 0) have_sizes = three_ints(value, dims);
    else if (key.rfind("data file", 0) == 0 || key.rfind("datafile", 0) == 0) data_file = value;
  }
  if (!have_sizes) return fail(err, "NRRD header without three positive sizes: " + path);
  if (data_file.empty()) return fail(err, "NRRD header without a detached 'data file': " + path);
  const int bpv = type.find("uint16") != std::string::npos ? 2 : 1;  // uint8 and anything else: 1 byte
  std::string name = path.substr(path.find_last_of("/\\") == std::string::npos ? 0 : path.find_last_of("/\\") + 1);
  *out = StructuredGridVolume(name, (int)dims[0], (int)dims[1], (int)dims[2]);
  out->SetScale(1.0, 1.0, 1.0);
  return read_raw_values(directory_of(path) + "/" + data_file, (int)dims[0], (int)dims[1], (int)dims[2], bpv, out,
                         err);
}

// readdat (reader.cpp:498-628).
bool read_dat(const std::string& path, StructuredGridVolume* out, std::string* err) {
  std::ifstream f(path);
  if (!f.is_open()) return fail(err, "opening .dat file failed: " + path);
  std::string line, key, value, object, format;
  long dims[3] = {0, 0, 0};
  double thick[3] = {1.0, 1.0, 1.0};
  bool have_res = false;
  while (std::getline(f, line)) {
    if (!key_value(line, &key, &value)) continue;
    if (key.rfind("ObjectFileName", 0) == 0) object = value;
    else if (key.rfind("Resolution", 0) == 0) have_res = three_ints(value, dims);
    else if (key.rfind("SliceThickness", 0) == 0) {
      std::istringstream is(value);
      double t[3];
      if (!(is >> t[0] >> t[1] >> t[2]) || !(t[0] > 0 && t[1] > 0 && t[2] > 0))
        return fail(err, "malformed SliceThickness '" + value + "': " + path);
      for (int k = 0; k < 3; ++k) thick[k] = (double)(float)t[k];  // glm::vec3
    } else if (key.rfind("Format", 0) == 0) {
      format = value;
    }
  }
  if (!have_res) return fail(err, ".dat without three positive Resolution values: " + path);
  if (object.empty()) return fail(err, ".dat without ObjectFileName: " + path);
  const int bpv = format.find("USHORT") != std::string::npos ? 2 : 1;  // UCHAR and anything else: 1 byte
  std::string name = path.substr(path.find_last_of("/\\") == std::string::npos ? 0 : path.find_last_of("/\\") + 1);
  *out = StructuredGridVolume(name, (int)dims[0], (int)dims[1], (int)dims[2]);
  out->SetScale(thick[0], thick[1], thick[2]);
  return read_raw_values(directory_of(path) + "/" + object, (int)dims[0], (int)dims[1], (int)dims[2], bpv, out, err);
}

}  // namespace

bool ReadPVM(const std::string& path, StructuredGridVolume* out, std::string* err) { return read_pvm(path, out, err); }
bool ReadNRRD(const std::string& path, StructuredGridVolume* out, std::string* err) {
  return read_nrrd(path, out, err);
}
bool ReadDAT(const std::string& path, StructuredGridVolume* out, std::string* err) { return read_dat(path, out, err); }

}  // namespace vis
