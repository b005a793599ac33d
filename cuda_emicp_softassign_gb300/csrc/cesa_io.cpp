// Point-cloud front end of the registration CLI (host code): the reference's
// loadFile (PLY through PCL, NaN points removed), pointsReduction,
// alignScaleOnce, saveRTtoFile and loadRTfromFile (src/main.cpp:41-228),
// restated without PCL.
//
//  - PLY: ASCII, binary little- and big-endian; the vertex element's x, y, z
//    properties of any scalar type; other properties and elements are skipped
//    (elements after the vertices are not read; a list property before them is
//    accepted in ASCII files only).
//  - PCD (PCL's format, which the reference's loadPolygonFile also reads):
//    DATA ascii, binary and binary_compressed (LZF, field-major); the first
//    element of the x, y and z fields of any F / I / U type.
//  - Text: "x y z ..." per line, '#' comments and blank lines skipped.
//  - Points with a non-finite coordinate are removed, as
//    pcl::removeNaNFromPointCloud does after loading.
//  - pointsReduction keeps each point with probability percent / 100 and
//    preserves the order; the reference draws from rand() seeded with the
//    clock (src/main.cpp:78-98), here the draw is a seeded SplitMix64 stream
//    so that runs repeat.
//  - alignScaleOnce scales each cloud about the origin by
//    sqrt(0.003 / trace(C)), C the covariance about the mean normalised by n
//    (src/main.cpp:124-161).
//  - The writers and the rigid transform serve the reference's point-cloud
//    tools (src/add_rigid_transform.cpp, src/merge.cpp, src/pcd2ply.cpp): PCD
//    as PCL's savePCDFileASCII writes it and ASCII PLY, both with 8
//    significant digits as PCL's writers use, and p' = R p + t in FP32.
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cesa.h"

namespace {

enum class PlyType { kInt8, kUInt8, kInt16, kUInt16, kInt32, kUInt32, kInt64, kUInt64, kFloat32, kFloat64, kBad };

PlyType ply_type(const std::string& s) {
  if (s == "char" || s == "int8") return PlyType::kInt8;
  if (s == "uchar" || s == "uint8") return PlyType::kUInt8;
  if (s == "short" || s == "int16") return PlyType::kInt16;
  if (s == "ushort" || s == "uint16") return PlyType::kUInt16;
  if (s == "int" || s == "int32") return PlyType::kInt32;
  if (s == "uint" || s == "uint32") return PlyType::kUInt32;
  if (s == "float" || s == "float32") return PlyType::kFloat32;
  if (s == "double" || s == "float64") return PlyType::kFloat64;
  return PlyType::kBad;
}

int type_size(PlyType t) {
  switch (t) {
    case PlyType::kInt8:
    case PlyType::kUInt8:
      return 1;
    case PlyType::kInt16:
    case PlyType::kUInt16:
      return 2;
    case PlyType::kInt32:
    case PlyType::kUInt32:
    case PlyType::kFloat32:
      return 4;
    case PlyType::kInt64:
    case PlyType::kUInt64:
    case PlyType::kFloat64:
      return 8;
    default:
      return 0;
  }
}

struct PlyProp {
  std::string name;
  PlyType type = PlyType::kBad;
  bool list = false;
  PlyType count_type = PlyType::kBad;
};

struct PlyElem {
  std::string name;
  long count = 0;
  std::vector<PlyProp> props;
};

bool host_little_endian() {
  const uint16_t v = 1;
  unsigned char b;
  std::memcpy(&b, &v, 1);
  return b == 1;
}

double decode(const unsigned char* p, PlyType t, bool swap) {
  unsigned char b[8];
  const int n = type_size(t);
  for (int i = 0; i < n; ++i) b[i] = swap ? p[n - 1 - i] : p[i];
  switch (t) {
    case PlyType::kInt8: {
      int8_t v;
      std::memcpy(&v, b, 1);
      return v;
    }
    case PlyType::kUInt8:
      return b[0];
    case PlyType::kInt16: {
      int16_t v;
      std::memcpy(&v, b, 2);
      return v;
    }
    case PlyType::kUInt16: {
      uint16_t v;
      std::memcpy(&v, b, 2);
      return v;
    }
    case PlyType::kInt32: {
      int32_t v;
      std::memcpy(&v, b, 4);
      return v;
    }
    case PlyType::kUInt32: {
      uint32_t v;
      std::memcpy(&v, b, 4);
      return v;
    }
    case PlyType::kInt64: {
      int64_t v;
      std::memcpy(&v, b, 8);
      return (double)v;
    }
    case PlyType::kUInt64: {
      uint64_t v;
      std::memcpy(&v, b, 8);
      return (double)v;
    }
    case PlyType::kFloat32: {
      float v;
      std::memcpy(&v, b, 4);
      return v;
    }
    case PlyType::kFloat64: {
      double v;
      std::memcpy(&v, b, 8);
      return v;
    }
    default:
      return 0.0;
  }
}

bool read_line(FILE* f, std::string& line) {
  line.clear();
  int c;
  while ((c = std::fgetc(f)) != EOF) {
    if (c == '\n') return true;
    if (c != '\r') line.push_back(static_cast<char>(c));
  }
  return !line.empty();
}

std::vector<std::string> split(const std::string& s) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < s.size()) {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\t')) ++i;
    size_t j = i;
    while (j < s.size() && s[j] != ' ' && s[j] != '\t') ++j;
    if (j > i) out.push_back(s.substr(i, j - i));
    i = j;
  }
  return out;
}

// Returns CESA_OK and appends x, y, z triples to pts.
int load_ply(FILE* f, std::vector<float>& pts) {
  std::string line;
  if (!read_line(f, line) || line != "ply") return CESA_ERR_INVALID_ARGUMENT;
  int format = -1;  // 0 ascii, 1 binary little endian, 2 binary big endian
  std::vector<PlyElem> elems;
  while (true) {
    if (!read_line(f, line)) return CESA_ERR_INVALID_ARGUMENT;
    const std::vector<std::string> w = split(line);
    if (w.empty()) continue;
    if (w[0] == "end_header") break;
    if (w[0] == "format" && w.size() >= 2) {
      if (w[1] == "ascii") format = 0;
      else if (w[1] == "binary_little_endian") format = 1;
      else if (w[1] == "binary_big_endian") format = 2;
      else return CESA_ERR_UNSUPPORTED;
    } else if (w[0] == "element" && w.size() >= 3) {
      PlyElem e;
      e.name = w[1];
      e.count = std::strtol(w[2].c_str(), nullptr, 10);
      if (e.count < 0) return CESA_ERR_INVALID_ARGUMENT;
      elems.push_back(e);
    } else if (w[0] == "property" && !elems.empty()) {
      PlyProp p;
      if (w.size() >= 5 && w[1] == "list") {
        p.list = true;
        p.count_type = ply_type(w[2]);
        p.type = ply_type(w[3]);
        p.name = w[4];
      } else if (w.size() >= 3) {
        p.type = ply_type(w[1]);
        p.name = w[2];
      } else {
        return CESA_ERR_INVALID_ARGUMENT;
      }
      if (p.type == PlyType::kBad || (p.list && p.count_type == PlyType::kBad)) return CESA_ERR_UNSUPPORTED;
      elems.back().props.push_back(p);
    }
    // comment, obj_info and unknown header lines are ignored
  }
  if (format < 0) return CESA_ERR_INVALID_ARGUMENT;
  const bool swap = (format == 1) != host_little_endian();
  for (const PlyElem& e : elems) {
    const bool vertex = e.name == "vertex";
    int ix = -1, iy = -1, iz = -1;
    bool has_list = false;
    for (size_t k = 0; k < e.props.size(); ++k) {
      if (e.props[k].name == "x") ix = (int)k;
      if (e.props[k].name == "y") iy = (int)k;
      if (e.props[k].name == "z") iz = (int)k;
      has_list = has_list || e.props[k].list;
    }
    if (vertex && (ix < 0 || iy < 0 || iz < 0)) return CESA_ERR_INVALID_ARGUMENT;
    if (format == 0) {
      for (long r = 0; r < e.count; ++r) {
        if (!read_line(f, line)) return CESA_ERR_INVALID_ARGUMENT;
        if (!vertex) continue;
        const std::vector<std::string> w = split(line);
        // scalar properties come first in order; a list property consumes its count + items
        double v[3] = {0, 0, 0};
        size_t pos = 0;
        for (size_t k = 0; k < e.props.size(); ++k) {
          if (pos >= w.size()) return CESA_ERR_INVALID_ARGUMENT;
          if (e.props[k].list) {
            const long c = std::strtol(w[pos].c_str(), nullptr, 10);
            pos += 1 + (size_t)(c > 0 ? c : 0);
            continue;
          }
          const double val = std::strtod(w[pos].c_str(), nullptr);
          if ((int)k == ix) v[0] = val;
          if ((int)k == iy) v[1] = val;
          if ((int)k == iz) v[2] = val;
          ++pos;
        }
        pts.push_back((float)v[0]);
        pts.push_back((float)v[1]);
        pts.push_back((float)v[2]);
      }
    } else {
      // variable-size records before (or in) the vertex element cannot be skipped
      if (has_list) return CESA_ERR_UNSUPPORTED;
      size_t rec = 0;
      std::vector<size_t> off(e.props.size());
      for (size_t k = 0; k < e.props.size(); ++k) {
        off[k] = rec;
        rec += (size_t)type_size(e.props[k].type);
      }
      std::vector<unsigned char> buf(rec);
      for (long r = 0; r < e.count; ++r) {
        if (rec && std::fread(buf.data(), 1, rec, f) != rec) return CESA_ERR_INVALID_ARGUMENT;
        if (!vertex) continue;
        pts.push_back((float)decode(buf.data() + off[ix], e.props[ix].type, swap));
        pts.push_back((float)decode(buf.data() + off[iy], e.props[iy].type, swap));
        pts.push_back((float)decode(buf.data() + off[iz], e.props[iz].type, swap));
      }
    }
    if (vertex) break;  // later elements (faces) are not needed
  }
  return CESA_OK;
}

int load_txt(FILE* f, std::vector<float>& pts) {
  std::string line;
  while (read_line(f, line)) {
    const std::vector<std::string> w = split(line);
    if (w.empty() || w[0][0] == '#') continue;
    if (w.size() < 3) return CESA_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < 3; ++k) {
      char* end = nullptr;
      const double v = std::strtod(w[k].c_str(), &end);
      if (end == w[k].c_str()) return CESA_ERR_INVALID_ARGUMENT;
      pts.push_back((float)v);
    }
  }
  return CESA_OK;
}

// ---- PCD -------------------------------------------------------------------

PlyType pcd_type(char t, int size) {
  if (t == 'F') return size == 4 ? PlyType::kFloat32 : size == 8 ? PlyType::kFloat64 : PlyType::kBad;
  if (t == 'I')
    return size == 1 ? PlyType::kInt8
           : size == 2 ? PlyType::kInt16
           : size == 4 ? PlyType::kInt32
           : size == 8 ? PlyType::kInt64
                       : PlyType::kBad;
  if (t == 'U')
    return size == 1 ? PlyType::kUInt8
           : size == 2 ? PlyType::kUInt16
           : size == 4 ? PlyType::kUInt32
           : size == 8 ? PlyType::kUInt64
                       : PlyType::kBad;
  return PlyType::kBad;
}

// LZF decompression (the liblzf stream format, used by PCD's
// binary_compressed data). A control byte c < 32 starts a literal run of
// c + 1 bytes. Otherwise c >> 5 is a length (7: add the next byte), the back
// reference is ((c & 31) << 8) + next byte + 1 bytes behind the output
// position, and length + 2 bytes are copied from there one at a time (the
// copy may overlap its own output). Returns the bytes written, or -1 when the
// stream is malformed or would overflow out.
long lzf_decompress(const unsigned char* in, size_t n_in, unsigned char* out, size_t n_out) {
  size_t ip = 0, op = 0;
  while (ip < n_in) {
    const unsigned c = in[ip++];
    if (c < 32) {
      const size_t len = (size_t)c + 1;
      if (ip + len > n_in || op + len > n_out) return -1;
      std::memcpy(out + op, in + ip, len);
      ip += len;
      op += len;
    } else {
      size_t len = c >> 5;
      if (len == 7) {
        if (ip >= n_in) return -1;
        len += in[ip++];
      }
      if (ip >= n_in) return -1;
      const size_t back = ((size_t)(c & 31) << 8) + in[ip++] + 1;
      len += 2;
      if (back > op || op + len > n_out) return -1;
      for (size_t k = 0; k < len; ++k, ++op) out[op] = out[op - back];
    }
  }
  return (long)op;
}

uint32_t read_u32le(const unsigned char* p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

// Returns CESA_OK and appends x, y, z triples to pts. Binary data is
// little-endian, as PCL writes it.
int load_pcd(FILE* f, std::vector<float>& pts) {
  std::vector<std::string> names;
  std::vector<int> sizes, counts;
  std::vector<char> types;
  long width = -1, height = 1, points = -1;
  int data = -1;  // 0 ascii, 1 binary, 2 binary_compressed
  std::string line;
  while (data < 0) {
    if (!read_line(f, line)) return CESA_ERR_INVALID_ARGUMENT;
    const std::vector<std::string> w = split(line);
    if (w.empty() || w[0][0] == '#') continue;
    const std::string& key = w[0];
    if (key == "FIELDS" || key == "COLUMNS") {
      names.assign(w.begin() + 1, w.end());
    } else if (key == "SIZE" || key == "COUNT") {
      std::vector<int>& v = key == "SIZE" ? sizes : counts;
      v.clear();
      for (size_t k = 1; k < w.size(); ++k) v.push_back((int)std::strtol(w[k].c_str(), nullptr, 10));
    } else if (key == "TYPE") {
      types.clear();
      for (size_t k = 1; k < w.size(); ++k) types.push_back(w[k][0]);
    } else if ((key == "WIDTH" || key == "HEIGHT" || key == "POINTS") && w.size() >= 2) {
      const long v = std::strtol(w[1].c_str(), nullptr, 10);
      (key == "WIDTH" ? width : key == "HEIGHT" ? height : points) = v;
    } else if (key == "DATA") {
      if (w.size() < 2) return CESA_ERR_INVALID_ARGUMENT;
      if (w[1] == "ascii") data = 0;
      else if (w[1] == "binary") data = 1;
      else if (w[1] == "binary_compressed") data = 2;
      else return CESA_ERR_UNSUPPORTED;
    }
    // VERSION, VIEWPOINT and unknown keys are ignored
  }
  const size_t nf = names.size();
  if (counts.empty()) counts.assign(nf, 1);
  if (nf == 0 || sizes.size() != nf || types.size() != nf || counts.size() != nf) return CESA_ERR_INVALID_ARGUMENT;
  if (points < 0 && width >= 0 && height >= 0) points = width * height;
  if (points < 0 || points > 0x7fffffffL) return CESA_ERR_INVALID_ARGUMENT;
  std::vector<PlyType> type(nf);
  std::vector<size_t> off(nf), tok(nf);
  size_t rec = 0, ntok = 0;
  int fx = -1, fy = -1, fz = -1;
  for (size_t k = 0; k < nf; ++k) {
    type[k] = pcd_type(types[k], sizes[k]);
    if (type[k] == PlyType::kBad) return CESA_ERR_UNSUPPORTED;
    if (counts[k] < 1 || counts[k] > (1 << 20)) return CESA_ERR_INVALID_ARGUMENT;
    off[k] = rec;
    tok[k] = ntok;
    rec += (size_t)sizes[k] * (size_t)counts[k];
    ntok += (size_t)counts[k];
    if (names[k] == "x") fx = (int)k;
    if (names[k] == "y") fy = (int)k;
    if (names[k] == "z") fz = (int)k;
  }
  if (fx < 0 || fy < 0 || fz < 0) return CESA_ERR_INVALID_ARGUMENT;
  const int fxyz[3] = {fx, fy, fz};
  const size_t np = (size_t)points;
  pts.reserve(pts.size() + 3 * np);
  if (data == 0) {
    for (size_t r = 0; r < np;) {
      if (!read_line(f, line)) return CESA_ERR_INVALID_ARGUMENT;
      const std::vector<std::string> w = split(line);
      if (w.empty()) continue;
      if (w.size() < ntok) return CESA_ERR_INVALID_ARGUMENT;
      for (int c = 0; c < 3; ++c) pts.push_back((float)std::strtod(w[tok[fxyz[c]]].c_str(), nullptr));
      ++r;
    }
    return CESA_OK;
  }
  const bool swap = !host_little_endian();
  if (data == 1) {
    std::vector<unsigned char> buf(rec);
    for (size_t r = 0; r < np; ++r) {
      if (std::fread(buf.data(), 1, rec, f) != rec) return CESA_ERR_INVALID_ARGUMENT;
      for (int c = 0; c < 3; ++c) pts.push_back((float)decode(buf.data() + off[fxyz[c]], type[fxyz[c]], swap));
    }
    return CESA_OK;
  }
  unsigned char sz[8];
  if (std::fread(sz, 1, 8, f) != 8) return CESA_ERR_INVALID_ARGUMENT;
  const size_t n_comp = read_u32le(sz), n_raw = read_u32le(sz + 4);
  if (n_raw != rec * np) return CESA_ERR_INVALID_ARGUMENT;
  std::vector<unsigned char> comp(n_comp), raw(n_raw);
  if (n_comp && std::fread(comp.data(), 1, n_comp, f) != n_comp) return CESA_ERR_INVALID_ARGUMENT;
  if (lzf_decompress(comp.data(), n_comp, raw.data(), n_raw) != (long)n_raw) return CESA_ERR_INVALID_ARGUMENT;
  // field-major: field k's values for all points start at np * off[k]
  for (size_t r = 0; r < np; ++r)
    for (int c = 0; c < 3; ++c) {
      const int k = fxyz[c];
      const size_t at = np * off[k] + r * (size_t)sizes[k] * (size_t)counts[k];
      pts.push_back((float)decode(raw.data() + at, type[k], swap));
    }
  return CESA_OK;
}

bool ends_with_ci(const char* s, const char* suffix) {
  const size_t n = std::strlen(s), m = std::strlen(suffix);
  if (m > n) return false;
  for (size_t i = 0; i < m; ++i) {
    char a = s[n - m + i];
    if (a >= 'A' && a <= 'Z') a = (char)(a - 'A' + 'a');
    if (a != suffix[i]) return false;
  }
  return true;
}

// %.8g as PCL's writers print (they print NaN as "nan")
void put8(FILE* f, float v, char sep) {
  if (std::isnan(v)) std::fprintf(f, "nan%c", sep);
  else std::fprintf(f, "%.8g%c", (double)v, sep);
}

uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// trace of the covariance about the mean, normalised by n (two passes in double)
double cov_trace(const float* p, int n) {
  double m[3] = {0, 0, 0};
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) m[k] += p[3 * i + k];
  for (int k = 0; k < 3; ++k) m[k] /= n;
  double s = 0;
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      const double d = p[3 * i + k] - m[k];
      s += d * d;
    }
  return s / n;
}

}  // namespace

extern "C" {

int cesa_load_points(const char* path, float** xyz, int* n) {
  if (!path || !xyz || !n) return CESA_ERR_INVALID_ARGUMENT;
  *xyz = nullptr;
  *n = 0;
  FILE* f = std::fopen(path, "rb");
  if (!f) return CESA_ERR_INVALID_ARGUMENT;
  char magic[7] = {0, 0, 0, 0, 0, 0, 0};
  const size_t got = std::fread(magic, 1, 6, f);
  std::rewind(f);
  std::vector<float> pts;
  const bool ply = got >= 3 && std::memcmp(magic, "ply", 3) == 0;
  const bool pcd = ends_with_ci(path, ".pcd") ||
                   (got == 6 && (std::memcmp(magic, "# .PCD", 6) == 0 || std::memcmp(magic, "VERSIO", 6) == 0));
  const int rc = ply ? load_ply(f, pts) : pcd ? load_pcd(f, pts) : load_txt(f, pts);
  std::fclose(f);
  if (rc != CESA_OK) return rc;
  // drop points with a non-finite coordinate
  size_t w = 0;
  for (size_t i = 0; i + 2 < pts.size(); i += 3) {
    if (std::isfinite(pts[i]) && std::isfinite(pts[i + 1]) && std::isfinite(pts[i + 2])) {
      pts[w] = pts[i];
      pts[w + 1] = pts[i + 1];
      pts[w + 2] = pts[i + 2];
      w += 3;
    }
  }
  if (w / 3 > 0x7fffffff) return CESA_ERR_UNSUPPORTED;
  float* out = static_cast<float*>(std::malloc(sizeof(float) * (w > 0 ? w : 3)));
  if (!out) return CESA_ERR_OUT_OF_MEMORY;
  if (w) std::memcpy(out, pts.data(), sizeof(float) * w);
  *xyz = out;
  *n = (int)(w / 3);
  return CESA_OK;
}

void cesa_free(void* p) { std::free(p); }

int cesa_points_reduction(float* xyz, int* n, float percent, unsigned long long seed) {
  if (!n || *n < 0 || (*n > 0 && !xyz) || !(percent >= 0.f)) return CESA_ERR_INVALID_ARGUMENT;
  const double keep = percent / 100.0;
  uint64_t s = seed;
  int w = 0;
  for (int i = 0; i < *n; ++i) {
    const double u = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);  // [0, 1)
    if (u < keep) {
      if (w != i)
        for (int k = 0; k < 3; ++k) xyz[3 * w + k] = xyz[3 * i + k];
      ++w;
    }
  }
  *n = w;
  return CESA_OK;
}

int cesa_align_scale_once(float* xyz1, int n1, float* xyz2, int n2) {
  if (n1 < 1 || n2 < 1 || !xyz1 || !xyz2) return CESA_ERR_INVALID_ARGUMENT;
  float* p[2] = {xyz1, xyz2};
  const int n[2] = {n1, n2};
  for (int c = 0; c < 2; ++c) {
    const double tr = cov_trace(p[c], n[c]);
    if (!(tr > 0.0)) return CESA_ERR_INVALID_ARGUMENT;
    const float s = (float)(1.0 / std::sqrt(tr) * std::sqrt(0.003));  // src/main.cpp:138-140
    for (int i = 0; i < 3 * n[c]; ++i) p[c][i] *= s;
  }
  return CESA_OK;
}

int cesa_save_rt(const char* path, const float R[9], const float t[3]) {
  if (!path || !R || !t) return CESA_ERR_INVALID_ARGUMENT;
  FILE* f = std::fopen(path, "w");
  if (!f) return CESA_ERR_INVALID_ARGUMENT;
  for (int r = 0; r < 9; ++r) {  // the reference's layout, src/main.cpp:197-211
    std::fprintf(f, "%f ", R[r]);
    if ((r + 1) % 3 == 0) std::fprintf(f, "\n");
  }
  for (int r = 0; r < 3; ++r) std::fprintf(f, "%f ", t[r]);
  std::fprintf(f, "\n");
  std::fclose(f);
  return CESA_OK;
}

int cesa_save_points(const char* path, const float* xyz, int n, int format) {
  if (!path || n < 0 || (n > 0 && !xyz) || format < CESA_POINTS_BY_NAME || format > CESA_POINTS_TEXT)
    return CESA_ERR_INVALID_ARGUMENT;
  if (format == CESA_POINTS_BY_NAME)
    format = ends_with_ci(path, ".pcd") ? CESA_POINTS_PCD : ends_with_ci(path, ".ply") ? CESA_POINTS_PLY
                                                                                       : CESA_POINTS_TEXT;
  FILE* f = std::fopen(path, "w");
  if (!f) return CESA_ERR_INVALID_ARGUMENT;
  const bool pcd = format == CESA_POINTS_PCD, ply = format == CESA_POINTS_PLY;
  if (pcd) {
    // the header PCL's savePCDFileASCII writes for a PointXYZ cloud of
    // height 1 with the default viewpoint
    std::fprintf(f,
                 "# .PCD v0.7 - Point Cloud Data file format\nVERSION 0.7\nFIELDS x y z\nSIZE 4 4 4\nTYPE F F F\n"
                 "COUNT 1 1 1\nWIDTH %d\nHEIGHT 1\nVIEWPOINT 0 0 0 1 0 0 0\nPOINTS %d\nDATA ascii\n",
                 n, n);
  } else if (ply) {
    std::fprintf(f,
                 "ply\nformat ascii 1.0\nelement vertex %d\nproperty float x\nproperty float y\n"
                 "property float z\nend_header\n",
                 n);
  }
  for (int i = 0; i < n; ++i) {
    const float* p = xyz + 3 * (size_t)i;
    if (pcd || ply) {
      put8(f, p[0], ' ');
      put8(f, p[1], ' ');
      put8(f, p[2], '\n');
    } else {
      std::fprintf(f, "%.9g %.9g %.9g\n", (double)p[0], (double)p[1], (double)p[2]);
    }
  }
  const bool ok = std::ferror(f) == 0;
  return (std::fclose(f) == 0 && ok) ? CESA_OK : CESA_ERR_INVALID_ARGUMENT;
}

int cesa_transform_points(float* xyz, int n, const float R[9], const float t[3]) {
  if (n < 0 || (n > 0 && !xyz) || !R || !t) return CESA_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < n; ++i) {
    float* p = xyz + 3 * (size_t)i;
    const float x = p[0], y = p[1], z = p[2];
    for (int r = 0; r < 3; ++r) {
      // each product and sum rounded in FP32, left to right (no fused
      // multiply-add: the library is built with -ffp-contract=off)
      const float a = R[3 * r] * x;
      const float b = R[3 * r + 1] * y;
      const float c = R[3 * r + 2] * z;
      p[r] = ((a + b) + c) + t[r];
    }
  }
  return CESA_OK;
}

int cesa_load_rt(const char* path, float R[9], float t[3]) {
  if (!path || !R || !t) return CESA_ERR_INVALID_ARGUMENT;
  FILE* f = std::fopen(path, "r");
  if (!f) return CESA_ERR_INVALID_ARGUMENT;
  float v[12];
  const int got = std::fscanf(f, "%f%f%f%f%f%f%f%f%f%f%f%f", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5], &v[6],
                              &v[7], &v[8], &v[9], &v[10], &v[11]);
  std::fclose(f);
  if (got != 12) return CESA_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < 9; ++i) R[i] = v[i];
  for (int i = 0; i < 3; ++i) t[i] = v[9 + i];
  return CESA_OK;
}

}  // extern "C"
