// CT-MHD 3D step kernels (in progress).
#pragma once
#include "ek_common.cuh"
namespace EK_NS
{
cudaError_t
mhd_dt(int, const void *, const KParams &, unsigned long long *, cudaStream_t)
{
  return cudaErrorNotSupported;
}
cudaError_t
mhd_step(int, const void *, void *, void *, const KParams &, DevClock *, int, cudaStream_t)
{
  return cudaErrorNotSupported;
}
size_t
mhd_work_bytes(int, const KParams &)
{
  return 0;
}
cudaError_t
mhd_divb_max(int, const void *, const KParams &, double *, cudaStream_t)
{
  return cudaErrorNotSupported;
}
} // namespace EK_NS
