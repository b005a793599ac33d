/*
 * Drop-in replacement for the reference's public header
 * (src/3dregistration.h): the same registrationParameters fields, in the same
 * order, and the same entry points emicp(), softassign(), emicp_cpu(), icp(),
 * findRTfromS(), printRT() and cloud2data(). Their implementation
 * (registration.cpp in the package's csrc/ directory) runs the GB300 kernels
 * of libcesa.so through the C ABI in cesa.h.
 *
 * With a real PCL installation this header includes PCL, like the reference.
 * Without one (or with CESA_NO_PCL defined) it uses the minimal PointXYZ /
 * PointCloud / shared_ptr stand-ins of cesa_pcl_compat.h.
 *
 * Differences from the reference, all on failure paths:
 *   - on an error, R and t keep their values on entry, and the reason is
 *     printed on stderr (the reference ignores CUDA errors,
 *     src/3dregistration.h:118);
 *   - the device is never reset (the reference calls cudaThreadExit,
 *     src/emicp.cu:713).
 */
#ifndef _3DREGISTRATION_H_
#define _3DREGISTRATION_H_

#if !defined(CESA_NO_PCL) && defined(__has_include)
#if __has_include(<pcl/visualization/cloud_viewer.h>)
#define CESA_HAVE_PCL 1
#endif
#endif

#ifdef CESA_HAVE_PCL
#include <pcl/common/transforms.h>
#include <pcl/visualization/cloud_viewer.h>
#else
#include "cesa_pcl_compat.h"
#endif

/* threads in a 2D block of the reference kernels (kept for source compatibility) */
#define BLOCK_SIZE 16

typedef struct {
  /* for softassign */
  int JMAX;       /* annealing steps, T <- T*TFACTOR after each (default 100) */
  int I0;         /* pose updates per temperature (default 5) */
  int I1;         /* Sinkhorn row/column passes per pose update (default 3) */
  float alpha;    /* outlier parameter (default 3.0) */
  float T_0;      /* initial temperature (default 100.0) */
  float TFACTOR;  /* temperature factor (default 0.95) */
  float moutlier; /* slack row/column initial value (default 1/sqrtf(T_0)*expf(-1.0f)) */

  /* for EM-ICP */
  float sigma_p2;     /* initial sigma_p^2 (default 0.01) */
  float sigma_inf;    /* final sigma_p^2 (default 0.00001) */
  float sigma_factor; /* sigma_p2 <- sigma_p2*sigma_factor (default 0.9) */
  float d_02;         /* outlier distance^2 (default 0.01) */

  /* for ICP */
  int maxIteration; /* default 30 */

  /* misc */
  int noviewer;
  int nostop;
  int notimer;

  int argc;
  char **argv;

  boost::shared_ptr<pcl::visualization::PCLVisualizer> viewer;
  pcl::visualization::PointCloudColorHandlerCustom<pcl::PointXYZ>::Ptr source_trans_color;
  pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_source;
  pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_source_trans;
  pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_target;
} registrationParameters;

/* X = cloud_target, Y = cloud_source; on return X ~ R*Y + t.
 * h_R: 9 floats row-major, h_t: 3 floats; initial pose on entry. */
void softassign(const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_target,
                const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_source, float *h_R, float *h_t,
                const registrationParameters &param);
void emicp(const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_target,
           const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_source, float *h_R, float *h_t,
           const registrationParameters &param);

/* The reference's CPU EM-ICP (src/emicp_cpu.cpp:186-547, declared at
 * src/3dregistration.h:91-95). This library has no CPU registration path: the
 * call runs the GPU EM-ICP of emicp() with the same parameters, and says so
 * once on stderr. Its result is emicp()'s. */
void emicp_cpu(const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_target,
               const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_source, float *h_R, float *h_t,
               const registrationParameters &param);

void icp(const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_target,
         const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_source, float *h_R, float *h_t,
         const registrationParameters &param);

void findRTfromS(const float *h_Xc, const float *h_Yc, const float *h_S, float *h_R, float *h_t);

/* Prints R (three rows) and t on stdout in the reference CLI's layout
 * (src/main.cpp:184-195, declared at src/3dregistration.h:111): a line "R",
 * three lines of three "%f " entries, a line "t", one line of three. */
void printRT(const float *R, const float *t);

void cloud2data(const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud, float **X, int &Xsize);
void cloud2data(const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud, boost::shared_array<float> &X,
                int &Xsize);

#define CUDA_SAFE_CALL(a) a
#define CUT_SAFE_CALL(a) a

#endif
