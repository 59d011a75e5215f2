// On-disk byte images -> native complex numbers on the device.
//
// The readers of lattice/filedata convert on the host after a memory map:
// ILDG gauge fields are stored big-endian and up-cast to complex128
// (lattice/filedata/ildg.py:70), QDP lazy-disk-map records are big-endian and
// cast to complex64 (lattice/filedata/timeslice.py:96), and the generators then
// transpose the links to [dir][t][z][y][x][3][3] (lattice/generator/elemental.py:103,
// eigenvector.py:50).  Here the stored bytes travel to HBM unchanged and one
// pass per array swaps the byte order, converts the precision and (for links)
// transposes.  Element-wise and HBM-bound: 16 (or 8) bytes read and 16 (or 8)
// written per complex number.
#include "common.cuh"

namespace ed {

namespace {

__device__ __forceinline__ uint32_t bswap32(uint32_t x) { return __byte_perm(x, 0u, 0x0123u); }

__device__ __forceinline__ unsigned long long bswap64(unsigned long long x) {
  const uint32_t lo = (uint32_t)x, hi = (uint32_t)(x >> 32);
  return ((unsigned long long)bswap32(lo) << 32) | bswap32(hi);
}

// Complex element i of a byte image: SRC16 = two 8-byte doubles, else two
// 4-byte floats; BE = stored big-endian.
template <bool SRC16, bool BE>
__device__ __forceinline__ double2 load_elem(const void* __restrict__ src, long long i) {
  if constexpr (SRC16) {
    ulonglong2 w = reinterpret_cast<const ulonglong2*>(src)[i];
    if constexpr (BE) {
      w.x = bswap64(w.x);
      w.y = bswap64(w.y);
    }
    return make_double2(__longlong_as_double((long long)w.x), __longlong_as_double((long long)w.y));
  } else {
    uint2 w = reinterpret_cast<const uint2*>(src)[i];
    if constexpr (BE) {
      w.x = bswap32(w.x);
      w.y = bswap32(w.y);
    }
    return make_double2((double)__uint_as_float(w.x), (double)__uint_as_float(w.y));
  }
}

template <bool DST16>
__device__ __forceinline__ void store_elem(void* __restrict__ dst, long long i, double2 v) {
  if constexpr (DST16)
    reinterpret_cast<double2*>(dst)[i] = v;
  else  // round to nearest, as numpy's astype to complex64
    reinterpret_cast<float2*>(dst)[i] = make_float2((float)v.x, (float)v.y);
}

template <bool SRC16, bool BE, bool DST16>
__global__ void decode_complex_kernel(const void* __restrict__ src, long long n, void* __restrict__ dst) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + stride < n; i += 2 * stride) {  // two loads in flight per thread
    const double2 a = load_elem<SRC16, BE>(src, i), b = load_elem<SRC16, BE>(src, i + stride);
    store_elem<DST16>(dst, i, a);
    store_elem<DST16>(dst, i + stride, b);
  }
  if (i < n) store_elem<DST16>(dst, i, load_elem<SRC16, BE>(src, i));
}

// dst [3][sites][9] complex128 <- src [sites][4][9] (the spatial directions
// of the ILDG site order).  Threads walk the source order (the 27 spatial
// elements of a site are contiguous, the 9 time-link elements skipped), so
// each warp reads one contiguous run and writes three runs of whole sites.
template <bool SRC16, bool BE>
__global__ void decode_links_kernel(const void* __restrict__ src, long long sites, double2* __restrict__ dst) {
  const long long n = 27 * sites;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long site = e / 27;
    const int r = (int)(e - site * 27), mu = r / 9, ab = r - 9 * (r / 9);
    dst[(long long)mu * sites * 9 + site * 9 + ab] = load_elem<SRC16, BE>(src, site * 36 + r);
  }
}

int grid_for(long long n) {
  const long long want = (n + 255) / 256, cap = 8LL * num_sms();
  return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

template <bool SRC16, bool BE>
void launch_decode(long long n, const void* src, bool dst16, void* dst, cudaStream_t s) {
  if (dst16)
    decode_complex_kernel<SRC16, BE, true><<<grid_for(n), 256, 0, s>>>(src, n, dst);
  else
    decode_complex_kernel<SRC16, BE, false><<<grid_for(n), 256, 0, s>>>(src, n, dst);
}

bool valid_src(int src_prec) {
  const int p = src_prec & ~ED_BIG_ENDIAN;
  return (src_prec & ~(ED_BIG_ENDIAN | 1)) == 0 && (p == ED_C128 || p == ED_C64);
}

}  // namespace

}  // namespace ed

extern "C" int ed_decode_complex(int src_prec, long long n, const void* src, int dst_prec, void* dst, void* stream) {
  using namespace ed;
  ED_CHECK_ARG(valid_src(src_prec), "ed_decode_complex: bad source precision %d", src_prec);
  ED_CHECK_ARG(dst_prec == ED_C128 || dst_prec == ED_C64, "ed_decode_complex: bad destination precision %d", dst_prec);
  ED_CHECK_ARG(n >= 0, "ed_decode_complex: negative count");
  if (n == 0) return ED_OK;
  ED_CHECK_ARG(src && dst, "ed_decode_complex: null pointer");
  const bool s16 = (src_prec & ~ED_BIG_ENDIAN) == ED_C128, be = (src_prec & ED_BIG_ENDIAN) != 0;
  const bool d16 = dst_prec == ED_C128;
  const size_t sz = s16 ? 16 : 8, dz = d16 ? 16 : 8;
  ED_CHECK_ARG((uintptr_t)src % sz == 0 && (uintptr_t)dst % dz == 0, "ed_decode_complex: misaligned pointer");
  const uintptr_t s0 = (uintptr_t)src, s1 = s0 + (uintptr_t)n * sz, d0 = (uintptr_t)dst, d1 = d0 + (uintptr_t)n * dz;
  ED_CHECK_ARG(s1 <= d0 || d1 <= s0, "ed_decode_complex: source and destination overlap");
  const cudaStream_t s = (cudaStream_t)stream;
  if (s16 && be)
    launch_decode<true, true>(n, src, d16, dst, s);
  else if (s16)
    launch_decode<true, false>(n, src, d16, dst, s);
  else if (be)
    launch_decode<false, true>(n, src, d16, dst, s);
  else
    launch_decode<false, false>(n, src, d16, dst, s);
  ED_RETURN_LAUNCH("ed_decode_complex");
  return ED_OK;
}

extern "C" int ed_decode_links(int src_prec, long long sites, const void* src, void* dst, void* stream) {
  using namespace ed;
  ED_CHECK_ARG(valid_src(src_prec), "ed_decode_links: bad source precision %d", src_prec);
  ED_CHECK_ARG(sites > 0, "ed_decode_links: sites must be positive");
  ED_CHECK_ARG(src && dst, "ed_decode_links: null pointer");
  const bool s16 = (src_prec & ~ED_BIG_ENDIAN) == ED_C128, be = (src_prec & ED_BIG_ENDIAN) != 0;
  const size_t sz = s16 ? 16 : 8;
  ED_CHECK_ARG((uintptr_t)src % sz == 0 && (uintptr_t)dst % 16 == 0, "ed_decode_links: misaligned pointer");
  const uintptr_t s0 = (uintptr_t)src, s1 = s0 + (uintptr_t)(sites * 36) * sz, d0 = (uintptr_t)dst,
                  d1 = d0 + (uintptr_t)(sites * 27) * 16;
  ED_CHECK_ARG(s1 <= d0 || d1 <= s0, "ed_decode_links: source and destination overlap");
  const cudaStream_t s = (cudaStream_t)stream;
  const int grid = grid_for(sites * 27);
  double2* out = (double2*)dst;
  if (s16 && be)
    decode_links_kernel<true, true><<<grid, 256, 0, s>>>(src, sites, out);
  else if (s16)
    decode_links_kernel<true, false><<<grid, 256, 0, s>>>(src, sites, out);
  else if (be)
    decode_links_kernel<false, true><<<grid, 256, 0, s>>>(src, sites, out);
  else
    decode_links_kernel<false, false><<<grid, 256, 0, s>>>(src, sites, out);
  ED_RETURN_LAUNCH("ed_decode_links");
  return ED_OK;
}
