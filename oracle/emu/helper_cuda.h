/* ORACLE / TEST INFRASTRUCTURE ONLY. The CUDA samples helper the reference
 * includes: device selection is a no-op on the host. */
#ifndef CESA_EMU_HELPER_CUDA_H_
#define CESA_EMU_HELPER_CUDA_H_
inline int findCudaDevice(int, const char**) { return 0; }
#endif
