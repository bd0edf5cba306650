// Device check of gch_convert.h, gch_ddiv.h and gch_dsqrt.h: the integer-pipe
// FP64 <-> FP32 conversions, FP64 division, FP64 square root and floor
// comparison, run in a kernel on the same cases as the host check
// (convert_cases.h), against the device's own IEEE operations in the same
// kernel: __ddiv_rn(a, b) for the division, __dsqrt_rn(x) for the square
// root, __double2float_rn(x) for FP64 -> FP32, the exact FP32 -> FP64
// conversion, and >= for the floor comparison, with the flush rule
// gch_convert.h states (results and FP32 inputs below 2^-126 in magnitude
// become signed zero).  The device quotients and roots are also compared with
// the host's IEEE operations.
// Usage: convert_check_gpu <n_random>; prints "checked N bad B", exits 1 on a
// mismatch and 2 on a CUDA error.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "convert_cases.h"
#include "gch_convert.h"
#include "gch_ddiv.h"
#include "gch_dsqrt.h"

__global__ void k_convert(const double* x, float* d2f_got, float* d2f_want,
                          unsigned char* ge_bad, long nx,
                          const float* f, double* f2d_got, double* f2d_want, long nf,
                          const double* a, const double* b, double* div_got, double* div_want,
                          long nd, const double* s, double* sq_got, double* sq_want, long ns) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nx; i += stride) {
    const double v = x[i];
    d2f_got[i] = gch::d2f_rn(v);
    d2f_want[i] = fabs(v) < 0x1p-126 ? copysignf(0.0f, (float)v) : __double2float_rn(v);
    // the integer-pipe floor comparison against the device's own, for the
    // pressure and density floors and 1
    unsigned m = 0;
    if (gch::ge_pos(v, 1e-16) != (v >= 1e-16)) m |= 1u;
    if (gch::ge_pos(v, 1e-15) != (v >= 1e-15)) m |= 2u;
    if (gch::ge_pos(v, 1.0) != (v >= 1.0)) m |= 4u;
    ge_bad[i] = (unsigned char)m;
  }
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += stride) {
    const float v = f[i];
    f2d_got[i] = gch::f2d(v);
    f2d_want[i] = ((__float_as_uint(v) >> 23) & 0xFFu) == 0 ? copysign(0.0, (double)v) : (double)v;
  }
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += stride) {
    div_got[i] = gch::ddiv_rn(a[i], b[i]);
    div_want[i] = __ddiv_rn(a[i], b[i]);
  }
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += stride) {
    sq_got[i] = gch::dsqrt_rn(s[i]);
    sq_want[i] = __dsqrt_rn(s[i]);
  }
}

#define CK(call)                                                                       \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      printf("CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return 2;                                                                        \
    }                                                                                  \
  } while (0)

template <class T>
static T* to_device(const std::vector<T>& h) {
  T* d = nullptr;
  if (cudaMalloc(&d, h.size() * sizeof(T) + 16) != cudaSuccess) return nullptr;
  if (cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
    return nullptr;
  return d;
}
template <class T>
static T* device_array(size_t n) {
  T* d = nullptr;
  if (cudaMalloc(&d, n * sizeof(T) + 16) != cudaSuccess) return nullptr;
  return d;
}
template <class T>
static bool same_bits(T got, T want) {
  return std::isnan(want) ? std::isnan(got) : gch::bits_of(got) == gch::bits_of(want);
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 200000;
  std::vector<double> xs, as, bs, ss;
  std::vector<float> fs;
  convert_cases(
      n, [&](double x) { xs.push_back(x); }, [&](float v) { fs.push_back(v); },
      [&](double a, double b) {
        as.push_back(a);
        bs.push_back(b);
      },
      [&](double v) { ss.push_back(v); });
  const long nx = (long)xs.size(), nf = (long)fs.size(), nd = (long)as.size(),
             ns = (long)ss.size();

  double *dx = to_device(xs), *da = to_device(as), *db = to_device(bs), *ds = to_device(ss);
  float* df = to_device(fs);
  float *d2f_got = device_array<float>(nx), *d2f_want = device_array<float>(nx);
  unsigned char* ge_bad = device_array<unsigned char>(nx);
  double *f2d_got = device_array<double>(nf), *f2d_want = device_array<double>(nf);
  double *div_got = device_array<double>(nd), *div_want = device_array<double>(nd);
  double *sq_got = device_array<double>(ns), *sq_want = device_array<double>(ns);
  if (!dx || !da || !db || !ds || !df || !d2f_got || !d2f_want || !ge_bad || !f2d_got ||
      !f2d_want || !div_got || !div_want || !sq_got || !sq_want) {
    printf("CUDA error: allocation or copy failed\n");
    return 2;
  }
  k_convert<<<4 * 152, 256>>>(dx, d2f_got, d2f_want, ge_bad, nx, df, f2d_got, f2d_want, nf,
                              da, db, div_got, div_want, nd, ds, sq_got, sq_want, ns);
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());

  std::vector<float> hg(nx), hw(nx);
  std::vector<unsigned char> gb(nx);
  std::vector<double> fg(nf), fw(nf), qg(nd), qw(nd), sg(ns), sw(ns);
  CK(cudaMemcpy(hg.data(), d2f_got, nx * sizeof(float), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hw.data(), d2f_want, nx * sizeof(float), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(gb.data(), ge_bad, nx * sizeof(unsigned char), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(fg.data(), f2d_got, nf * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(fw.data(), f2d_want, nf * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(qg.data(), div_got, nd * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(qw.data(), div_want, nd * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(sg.data(), sq_got, ns * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(sw.data(), sq_want, ns * sizeof(double), cudaMemcpyDeviceToHost));

  long checked = 0, bad = 0;
  for (long i = 0; i < nx; ++i, ++checked)
    if (!same_bits(hg[i], hw[i]) && bad++ < 8)
      printf("device d2f_rn(%a) = %a, device conversion %a\n", xs[i], hg[i], hw[i]);
  for (long i = 0; i < nx; ++i, ++checked)
    if (gb[i] && bad++ < 8)
      printf("device ge_pos(%a, floor) differs from >= (floor mask %u)\n", xs[i], (unsigned)gb[i]);
  for (long i = 0; i < nf; ++i, ++checked)
    if (!same_bits(fg[i], fw[i]) && bad++ < 8)
      printf("device f2d(%a) = %a, device conversion %a\n", fs[i], fg[i], fw[i]);
  for (long i = 0; i < nd; ++i, ++checked) {
    const double host = as[i] / bs[i];
    if ((!same_bits(qg[i], qw[i]) || !same_bits(qg[i], host)) && bad++ < 8)
      printf("device ddiv_rn(%a, %a) = %a, device division %a, host %a\n", as[i], bs[i], qg[i],
             qw[i], host);
  }
  for (long i = 0; i < ns; ++i, ++checked) {
    const double host = std::sqrt(ss[i]);
    if ((!same_bits(sg[i], sw[i]) || !same_bits(sg[i], host)) && bad++ < 8)
      printf("device dsqrt_rn(%a) = %a, device square root %a, host %a\n", ss[i], sg[i], sw[i],
             host);
  }
  printf("checked %ld bad %ld\n", checked, bad);
  return bad ? 1 : 0;
}
