/*
 * Minimal stand-ins for the three PCL / Boost types that the registration
 * API names in its signatures, for programs built without PCL:
 *
 *   pcl::PointXYZ                          x, y, z floats (padded to 16 bytes as in PCL)
 *   pcl::PointCloud<PointT>                .points vector, size(), ::Ptr
 *   pcl::visualization::PCLVisualizer      opaque (the viewer is not built)
 *   pcl::visualization::PointCloudColorHandlerCustom<PointT>::Ptr
 *   boost::shared_ptr / boost::shared_array
 *
 * When a real PCL installation is visible (<pcl/point_cloud.h> exists), the
 * drop-in header uses PCL itself and this file is not included.
 */
#ifndef CESA_PCL_COMPAT_H_
#define CESA_PCL_COMPAT_H_

#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

namespace boost {
template <class T>
using shared_ptr = std::shared_ptr<T>;

/* Owning pointer to a new[]-allocated array, released with delete[]. */
template <class T>
class shared_array {
 public:
  shared_array() = default;
  explicit shared_array(T* p) { reset(p); }
  void reset(T* p = nullptr) { p_.reset(p, [](T* q) { delete[] q; }); }
  T* get() const { return p_.get(); }
  T& operator[](std::ptrdiff_t i) const { return p_.get()[i]; }
  explicit operator bool() const { return static_cast<bool>(p_); }

 private:
  std::shared_ptr<T> p_;
};
}  // namespace boost

namespace pcl {
struct PointXYZ {
  float x = 0.f, y = 0.f, z = 0.f;
  float pad_ = 1.f; /* PCL stores points as 4 floats (x, y, z, 1) */
  PointXYZ() = default;
  PointXYZ(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
};

template <class PointT>
class PointCloud {
 public:
  typedef boost::shared_ptr<PointCloud<PointT> > Ptr;
  typedef boost::shared_ptr<const PointCloud<PointT> > ConstPtr;
  std::vector<PointT> points;
  uint32_t width = 0;
  uint32_t height = 1;
  bool is_dense = true;
  std::size_t size() const { return points.size(); }
  bool empty() const { return points.empty(); }
  void push_back(const PointT& p) {
    points.push_back(p);
    width = static_cast<uint32_t>(points.size());
  }
};

namespace visualization {
class PCLVisualizer {};
template <class PointT>
class PointCloudColorHandlerCustom {
 public:
  typedef boost::shared_ptr<PointCloudColorHandlerCustom<PointT> > Ptr;
};
}  // namespace visualization
}  // namespace pcl

#endif /* CESA_PCL_COMPAT_H_ */
