// The reference's point-cloud tools over libcesa.so's front end, without PCL:
//
//   add_rigid_transform <in> <out> <RT file>   out = R in + t
//                                              (src/add_rigid_transform.cpp:89-113)
//   merge <in1> <in2> <out>                    out = in1's points, then in2's
//                                              (src/merge.cpp:58-77)
//   pcd2ply <in> <out>                         out = in, as ASCII PLY
//                                              (src/pcd2ply.cpp:57-70)
//
// Inputs are PLY, PCD or text (cesa_load_points, which drops non-finite points
// as the reference's loadFile does). add_rigid_transform and merge write
// ASCII PCD as PCL's savePCDFileASCII does, or ASCII PLY when the output name
// ends in .ply (the *_ply variants the bunny-building demo targets call,
// Makefile.demo:108-137). The RT file is the registration CLI's
// (cesa_load_rt). One executable serves the three tools: it picks the tool by
// the name it runs under, or by a first argument naming the tool.
//
// Unlike the reference, a missing argument, an unreadable input or RT file,
// or a failed write prints a message and exits 1 (the reference goes on with
// an empty cloud or an uninitialised pose).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cesa.h"

namespace {

std::string base_name(const char* p) {
  const char* s = std::strrchr(p, '/');
  return s ? s + 1 : p;
}

bool load(const char* path, std::vector<float>& pts) {
  float* xyz = nullptr;
  int n = 0;
  const int rc = cesa_load_points(path, &xyz, &n);
  if (rc != CESA_OK) {
    std::fprintf(stderr, "loadFile failed [%s]: %s\n", path, cesa_status_string(rc));
    return false;
  }
  pts.assign(xyz, xyz + 3 * (size_t)n);
  cesa_free(xyz);
  return true;
}

// ASCII PLY for a .ply name, else ASCII PCD (whatever the name, as PCL's
// savePCDFileASCII)
int by_name(const char* path) {
  const size_t n = std::strlen(path);
  return n >= 4 && (std::strcmp(path + n - 4, ".ply") == 0 || std::strcmp(path + n - 4, ".PLY") == 0)
             ? CESA_POINTS_PLY
             : CESA_POINTS_PCD;
}

int save(const char* path, const std::vector<float>& pts, int format) {
  const int rc = cesa_save_points(path, pts.data(), (int)(pts.size() / 3), format);
  if (rc != CESA_OK) {
    std::fprintf(stderr, "cannot write [%s]: %s\n", path, cesa_status_string(rc));
    return 1;
  }
  return 0;
}

int add_rigid_transform(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: add_rigid_transform <in> <out> <RT file>\n");
    return 1;
  }
  std::vector<float> pts;
  if (!load(argv[1], pts)) return 1;
  float R[9], t[3];
  if (cesa_load_rt(argv[3], R, t) != CESA_OK) {
    std::fprintf(stderr, "Fail to read RT from file [%s]\n", argv[3]);
    return 1;
  }
  cesa_transform_points(pts.data(), (int)(pts.size() / 3), R, t);
  return save(argv[2], pts, by_name(argv[2]));
}

int merge(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: merge <in1> <in2> <out>\n");
    return 1;
  }
  std::vector<float> a, b;
  if (!load(argv[1], a) || !load(argv[2], b)) return 1;
  a.insert(a.end(), b.begin(), b.end());
  return save(argv[3], a, by_name(argv[3]));
}

int pcd2ply(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: pcd2ply <in> <out>\n");
    return 1;
  }
  std::vector<float> pts;
  if (!load(argv[1], pts)) return 1;
  return save(argv[2], pts, CESA_POINTS_PLY);
}

int dispatch(const std::string& tool, int argc, char** argv) {
  if (tool == "add_rigid_transform" || tool == "add_rigid_transform_ply") return add_rigid_transform(argc, argv);
  if (tool == "merge" || tool == "merge_ply") return merge(argc, argv);
  if (tool == "pcd2ply") return pcd2ply(argc, argv);
  return -1;
}

}  // namespace

int main(int argc, char** argv) {
  int rc = dispatch(base_name(argv[0]), argc, argv);
  if (rc < 0 && argc >= 2) rc = dispatch(argv[1], argc - 1, argv + 1);
  if (rc < 0) {
    std::fprintf(stderr, "usage: %s add_rigid_transform|merge|pcd2ply <args>\n", argv[0]);
    return 1;
  }
  return rc;
}
