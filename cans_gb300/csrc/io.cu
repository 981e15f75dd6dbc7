// Restart checkpoints in the reference's binary format (src/load.f90:461-589,
// load_one_mpiio): one file per variable (fld_u.bin, fld_v.bin, fld_w.bin, fld_p.bin in
// src/main.f90:383,603-615) holding the interior of the field in Fortran order, FP64,
// native byte order, followed by the two FP64 values [time, istep].  A file whose size is
// not (ng1*ng2*ng3 + 2) * 8 bytes is rejected (the reference stops the run).
//
// Device side: the interior of the haloed field is packed into (or unpacked from) a
// contiguous device buffer by one kernel, and moved with one cudaMemcpy per file.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "cans_internal.cuh"

namespace {
constexpr int kTB = 256;

__global__ void k_pack(const double *__restrict__ p, double *__restrict__ out, int n1, int n2, int n3) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long nx = n1, ny = n2;
  if (t >= nx * ny * n3) return;
  const int i = (int)(t % nx) + 1, j = (int)((t / nx) % ny) + 1, k = (int)(t / (nx * ny)) + 1;
  out[t] = p[hidx(i, j, k, n1, n2)];
}

__global__ void k_unpack(const double *__restrict__ in, double *__restrict__ p, int n1, int n2, int n3) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long nx = n1, ny = n2;
  if (t >= nx * ny * n3) return;
  const int i = (int)(t % nx) + 1, j = (int)((t / nx) % ny) + 1, k = (int)(t / (nx * ny)) + 1;
  p[hidx(i, j, k, n1, n2)] = in[t];
}

struct DevBuf {
  double *d = nullptr;
  ~DevBuf() { cudaFree(d); }
};
}  // namespace

extern "C" int cans_save_field(const char *path, const int n[3], const double *p, double time, int istep,
                               void *stream) {
  if (!path || !n || !p || n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  const size_t np = (size_t)n[0] * n[1] * n[2];
  cudaStream_t st = as_stream(stream);
  DevBuf buf;
  CANS_CUDA_TRY(cudaMalloc(&buf.d, np * sizeof(double)));
  k_pack<<<(unsigned)((np + kTB - 1) / kTB), kTB, 0, st>>>(p, buf.d, n[0], n[1], n[2]);
  CANS_LAUNCH_CHECK();
  std::vector<double> h(np + 2);
  CANS_CUDA_TRY(cudaMemcpyAsync(h.data(), buf.d, np * sizeof(double), cudaMemcpyDeviceToHost, st));
  CANS_CUDA_TRY(cudaStreamSynchronize(st));
  h[np] = time;
  h[np + 1] = 1. * istep;  // fldinfo = [time, 1._rp*istep]
  FILE *f = fopen(path, "wb");
  if (!f) return CANS_EIO;
  const size_t w = fwrite(h.data(), sizeof(double), h.size(), f);
  const int cl = fclose(f);
  return (w == h.size() && cl == 0) ? CANS_OK : CANS_EIO;
}

extern "C" int cans_load_field(const char *path, const int n[3], double *p, double *time, int *istep,
                               void *stream) {
  if (!path || !n || !p || n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  const size_t np = (size_t)n[0] * n[1] * n[2];
  FILE *f = fopen(path, "rb");
  if (!f) return CANS_EIO;
  long long size = -1;
  if (fseek(f, 0, SEEK_END) == 0) size = (long long)ftell(f);
  if (size != (long long)((np + 2) * sizeof(double))) {
    fclose(f);
    return CANS_EINVAL;  // checkpoint of a different grid, or truncated
  }
  std::vector<double> h(np + 2);
  const bool ok = fseek(f, 0, SEEK_SET) == 0 && fread(h.data(), sizeof(double), h.size(), f) == h.size();
  fclose(f);
  if (!ok) return CANS_EIO;
  cudaStream_t st = as_stream(stream);
  DevBuf buf;
  CANS_CUDA_TRY(cudaMalloc(&buf.d, np * sizeof(double)));
  CANS_CUDA_TRY(cudaMemcpyAsync(buf.d, h.data(), np * sizeof(double), cudaMemcpyHostToDevice, st));
  k_unpack<<<(unsigned)((np + kTB - 1) / kTB), kTB, 0, st>>>(buf.d, p, n[0], n[1], n[2]);
  CANS_LAUNCH_CHECK();
  CANS_CUDA_TRY(cudaStreamSynchronize(st));
  if (time) *time = h[np];
  if (istep) *istep = (int)llround(h[np + 1]);  // istep = nint(fldinfo(2))
  return CANS_OK;
}
