// Error state, layout conversions and momentum-phase tables.
#include <cstdarg>
#include <cstring>
#include <algorithm>
#include <vector>

#include "common.cuh"

namespace ed {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

int cuda_status(cudaError_t e, const char* what) {
  set_error("%s: CUDA error %d (%s)", what, (int)e, cudaGetErrorString(e));
  return ED_ERR_CUDA;
}

// ------------------------------------------------------------ links
template <typename TO>
__global__ void links_to_soa_kernel(int V3, int nt, const cplx<double>* __restrict__ in, long long t_stride,
                                    long long dir_stride, long long site_stride, cplx<TO>* __restrict__ out) {
  // one thread per (t, site); writes 27 planes, each access coalesced on the output side
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)V3 * nt) return;
  const int t = (int)(idx / V3);
  const int s = (int)(idx - (long long)t * V3);
  cplx<TO>* o = out + (long long)t * 27 * V3 + s;
#pragma unroll
  for (int mu = 0; mu < 3; ++mu) {
    const cplx<double>* p = in + t * t_stride + mu * dir_stride + (long long)s * site_stride;
#pragma unroll
    for (int e = 0; e < 9; ++e) o[(mu * 9 + e) * V3] = cvt<TO>(ld(p + e));
  }
}

// ------------------------------------------------------------ vectors
template <typename TI, typename TO>
__global__ void to_planes_kernel(long long nvec, int V3, int round_c64, const cplx<TI>* __restrict__ in,
                                 cplx<TO>* __restrict__ out) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nvec * V3) return;
  const long long v = idx / V3;
  const int s = (int)(idx - v * V3);
  const cplx<TI>* p = in + (v * V3 + s) * 3;
  cplx<TO>* o = out + v * 3 * V3 + s;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    cplx<TI> a = p[c];
    if (round_c64) a = cvt<TI>(cvt<float>(a));
    o[c * V3] = cvt<TO>(a);
  }
}

template <typename TI, typename TO>
__global__ void from_planes_kernel(long long nvec, int V3, const cplx<TI>* __restrict__ in,
                                   cplx<TO>* __restrict__ out) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nvec * V3) return;
  const long long v = idx / V3;
  const int s = (int)(idx - v * V3);
  const cplx<TI>* p = in + v * 3 * V3 + s;
  cplx<TO>* o = out + (v * V3 + s) * 3;
#pragma unroll
  for (int c = 0; c < 3; ++c) o[c] = cvt<TO>(p[c * V3]);
}

// ------------------------------------------------------------ phases
struct MomTable {
  int n;
  int p[64][3];
};

// exp(+2 pi i (px x/Lx + py y/Ly + pz z/Lz)).  The angle is reduced exactly
// in integers (numerator over Lx*Ly*Lz, modulo 2*Lx*Ly*Lz), then sincospi.
__global__ void phase_kernel(Latt L, MomTable mt, int m0, cplx<double>* __restrict__ out) {
  const int V3 = L.V3();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = blockIdx.y;
  if (s >= V3 || m >= mt.n) return;
  const int x = s % L.Lx, y = (s / L.Lx) % L.Ly, z = s / (L.Lx * L.Ly);
  const long long D = (long long)V3;  // common denominator Lx*Ly*Lz
  long long num = 2LL * ((long long)mt.p[m][0] * x * L.Ly * L.Lz + (long long)mt.p[m][1] * y * L.Lx * L.Lz +
                         (long long)mt.p[m][2] * z * L.Lx * L.Ly);
  num %= 2 * D;
  if (num < 0) num += 2 * D;
  double sn, cs;
  sincospi((double)num / (double)D, &sn, &cs);
  out[(long long)(m0 + m) * V3 + s] = mk(cs, sn);
}

int launch_phases(Latt L, const int* moms, int nmom, cplx<double>* out, cudaStream_t stream) {
  const int V3 = L.V3();
  for (int m0 = 0; m0 < nmom; m0 += 64) {
    MomTable mt;
    mt.n = nmom - m0 < 64 ? nmom - m0 : 64;
    for (int i = 0; i < mt.n; ++i)
      for (int k = 0; k < 3; ++k) mt.p[i][k] = moms[(m0 + i) * 3 + k];
    dim3 grid(ceil_div(V3, 256), mt.n);
    phase_kernel<<<grid, 256, 0, stream>>>(L, mt, m0, out);
    ED_RETURN_LAUNCH("momentum phases");
  }
  return ED_OK;
}

int launch_links_to_soa(int out_prec, Latt L, int nt, const void* in, long long ts, long long ds, long long ss,
                        void* out, cudaStream_t stream) {
  const long long n = (long long)L.V3() * nt;
  const int grid = ceil_div(n, 256);
  if (out_prec == ED_C128)
    links_to_soa_kernel<double><<<grid, 256, 0, stream>>>(L.V3(), nt, (const cplx<double>*)in, ts, ds, ss,
                                                          (cplx<double>*)out);
  else
    links_to_soa_kernel<float><<<grid, 256, 0, stream>>>(L.V3(), nt, (const cplx<double>*)in, ts, ds, ss,
                                                         (cplx<float>*)out);
  ED_RETURN_LAUNCH("links to SoA");
  return ED_OK;
}

int launch_to_planes(int ip, int op, int round_c64, long long nvec, int V3, const void* in, void* out,
                     cudaStream_t stream) {
  const int grid = ceil_div(nvec * V3, 256);
  if (ip == ED_C128 && op == ED_C128)
    to_planes_kernel<double, double><<<grid, 256, 0, stream>>>(nvec, V3, round_c64, (const cplx<double>*)in,
                                                               (cplx<double>*)out);
  else if (ip == ED_C128 && op == ED_C64)
    to_planes_kernel<double, float><<<grid, 256, 0, stream>>>(nvec, V3, round_c64, (const cplx<double>*)in,
                                                              (cplx<float>*)out);
  else if (ip == ED_C64 && op == ED_C128)
    to_planes_kernel<float, double><<<grid, 256, 0, stream>>>(nvec, V3, round_c64, (const cplx<float>*)in,
                                                              (cplx<double>*)out);
  else
    to_planes_kernel<float, float><<<grid, 256, 0, stream>>>(nvec, V3, round_c64, (const cplx<float>*)in,
                                                             (cplx<float>*)out);
  ED_RETURN_LAUNCH("vectors to planes");
  return ED_OK;
}

int launch_from_planes(int ip, int op, long long nvec, int V3, const void* in, void* out, cudaStream_t stream) {
  const int grid = ceil_div(nvec * V3, 256);
  if (ip == ED_C128 && op == ED_C128)
    from_planes_kernel<double, double><<<grid, 256, 0, stream>>>(nvec, V3, (const cplx<double>*)in,
                                                                 (cplx<double>*)out);
  else if (ip == ED_C128 && op == ED_C64)
    from_planes_kernel<double, float><<<grid, 256, 0, stream>>>(nvec, V3, (const cplx<double>*)in,
                                                                (cplx<float>*)out);
  else if (ip == ED_C64 && op == ED_C128)
    from_planes_kernel<float, double><<<grid, 256, 0, stream>>>(nvec, V3, (const cplx<float>*)in,
                                                                (cplx<double>*)out);
  else
    from_planes_kernel<float, float><<<grid, 256, 0, stream>>>(nvec, V3, (const cplx<float>*)in,
                                                               (cplx<float>*)out);
  ED_RETURN_LAUNCH("vectors from planes");
  return ED_OK;
}

}  // namespace ed

// ------------------------------------------------------------ C ABI

extern "C" int ed_version(void) { return 100; }

extern "C" int ed_last_error(char* buf, size_t len) {
  const std::string& s = ed::g_last_error;
  if (buf && len > 0) {
    size_t n = s.size() < len - 1 ? s.size() : len - 1;
    memcpy(buf, s.data(), n);
    buf[n] = 0;
  }
  return (int)s.size();
}

static bool valid_prec(int p) { return p == ED_C128 || p == ED_C64; }

extern "C" int ed_links_to_soa(int out_prec, int Lx, int Ly, int Lz, int nt, const void* in, long long t_stride,
                               long long dir_stride, long long site_stride, void* out, void* stream) {
  ED_CHECK_ARG(valid_prec(out_prec), "ed_links_to_soa: bad precision");
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && nt > 0, "ed_links_to_soa: sizes must be positive");
  ED_CHECK_ARG(ed::lattice_ok(Lx, Ly, Lz), "ed_links_to_soa: Lx*Ly*Lz above 2^28");
  ED_CHECK_ARG(in && out, "ed_links_to_soa: null pointer");
  ED_CHECK_ARG(t_stride >= 0 && dir_stride >= 0 && site_stride >= 0, "ed_links_to_soa: negative stride");
  return ed::launch_links_to_soa(out_prec, ed::Latt{Lx, Ly, Lz}, nt, in, t_stride, dir_stride, site_stride, out,
                                 (cudaStream_t)stream);
}

extern "C" int ed_vectors_to_planes(int in_prec, int out_prec, int round_c64, long long nvec, int V3,
                                    const void* in, void* out, void* stream) {
  ED_CHECK_ARG(valid_prec(in_prec) && valid_prec(out_prec), "ed_vectors_to_planes: bad precision");
  ED_CHECK_ARG(nvec > 0 && V3 > 0, "ed_vectors_to_planes: sizes must be positive");
  ED_CHECK_ARG(in && out && in != out, "ed_vectors_to_planes: null or aliasing pointers");
  return ed::launch_to_planes(in_prec, out_prec, round_c64, nvec, V3, in, out, (cudaStream_t)stream);
}

extern "C" int ed_vectors_from_planes(int in_prec, int out_prec, long long nvec, int V3, const void* in, void* out,
                                      void* stream) {
  ED_CHECK_ARG(valid_prec(in_prec) && valid_prec(out_prec), "ed_vectors_from_planes: bad precision");
  ED_CHECK_ARG(nvec > 0 && V3 > 0, "ed_vectors_from_planes: sizes must be positive");
  ED_CHECK_ARG(in && out && in != out, "ed_vectors_from_planes: null or aliasing pointers");
  return ed::launch_from_planes(in_prec, out_prec, nvec, V3, in, out, (cudaStream_t)stream);
}

extern "C" int ed_momentum_phases(int Lx, int Ly, int Lz, const int* moms, int nmom, void* out, void* stream) {
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && nmom > 0, "ed_momentum_phases: sizes must be positive");
  ED_CHECK_ARG(ed::lattice_ok(Lx, Ly, Lz), "ed_momentum_phases: Lx*Ly*Lz above 2^28");
  ED_CHECK_ARG(moms && out, "ed_momentum_phases: null pointer");
  ED_CHECK_ARG((long long)Lx * Ly * Lz * 2 * 64 < (1LL << 52), "ed_momentum_phases: lattice too large");
  for (int i = 0; i < 3 * nmom; ++i)
    ED_CHECK_ARG(moms[i] > -1000000 && moms[i] < 1000000, "ed_momentum_phases: momentum component out of range");
  return ed::launch_phases(ed::Latt{Lx, Ly, Lz}, moms, nmom, (ed::cplx<double>*)out, (cudaStream_t)stream);
}

// ------------------------------------------------------------ mean of arrays
namespace ed {
__global__ void mean_kernel(int nsrc, long long n, long long src_stride, const cplx<double>* __restrict__ src,
                            cplx<double>* __restrict__ out) {
  const double inv = 1.0 / nsrc;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double re = 0.0, im = 0.0;
    for (int k = 0; k < nsrc; ++k) {
      const cplx<double> v = src[k * src_stride + i];
      re += v.re;
      im += v.im;
    }
    out[i] = mk(re * inv, im * inv);
  }
}
}  // namespace ed

extern "C" int ed_mean_c128(int nsrc, long long n, long long src_stride, const void* src, void* out, void* stream) {
  ED_CHECK_ARG(nsrc > 0 && n > 0 && src_stride >= n, "ed_mean_c128: bad sizes");
  ED_CHECK_ARG(src && out, "ed_mean_c128: null pointer");
  const int grid = (int)std::min<long long>(ed::ceil_div(n, 256), 8LL * ed::num_sms());
  ed::mean_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(nsrc, n, src_stride, (const ed::cplx<double>*)src,
                                                          (ed::cplx<double>*)out);
  ED_RETURN_LAUNCH("mean");
  return ED_OK;
}
