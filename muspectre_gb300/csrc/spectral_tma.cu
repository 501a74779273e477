// TMA-fed Green pass (FP32): the kernels of spectral_tma.cuh, their tensor-map
// descriptors and launcher, and the device fault word of their bounded waits.
#include <cstring>
#include <map>
#include <tuple>

#include "spectral_launch.cuh"
#include "spectral_tma.cuh"

namespace musg {

void wait_probe(unsigned long long limit_ns, cudaStream_t s) {
  k_wait_probe<<<1, 32, 0, s>>>(limit_ns);
  MUSG_CHECK_LAUNCH();
}

unsigned *wait_fault_word() {
  static unsigned *p = [] {
    void *q = nullptr;
    MUSG_CUDA(cudaGetSymbolAddress(&q, g_wait_fault));
    return static_cast<unsigned *>(q);
  }();
  return p;
}

namespace {

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver through the runtime's entry-point query
// (no link against the driver library); null when the driver does not offer it
EncodeTiledFn encode_tiled_fn() {
  static EncodeTiledFn fn = []() -> EncodeTiledFn {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      (void)cudaGetLastError();
      return nullptr;
    }
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

using GreenTmaKernel = void (*)(const GreenArgs<float>, const CUtensorMap);

template <int MODE, int D, int TT> GreenTmaKernel green_tma_kernel(int m) {
  switch (m) {
    case 16: return k_green_tma<16, MODE, D, TT>;
    case 32: return k_green_tma<32, MODE, D, TT>;
    case 64: return k_green_tma<64, MODE, D, TT>;
    case 128: return k_green_tma<128, MODE, D, TT>;
    case 256: return k_green_tma<256, MODE, D, TT>;
    default: return nullptr;
  }
}

template <int TT> GreenTmaKernel green_tma_kernel(int mode, int dim, int m) {
  if (mode == GM_FINITE) return dim == 2 ? green_tma_kernel<GM_FINITE, 2, TT>(m) : green_tma_kernel<GM_FINITE, 3, TT>(m);
  return dim == 2 ? green_tma_kernel<GM_SMALL, 2, TT>(m) : green_tma_kernel<GM_SMALL, 3, TT>(m);
}

// resident blocks per SM x SMs for a kernel launch shape (cached; thread-safe)
int persistent_grid(const void *k, int threads, size_t smem) {
  static std::mutex mu;
  static std::map<std::tuple<const void *, int, size_t>, int> cache;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_tuple(k, threads, smem);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int per_sm = 0, dev = 0, nsm = 0;
  MUSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem));
  MUSG_CUDA(cudaGetDevice(&dev));
  MUSG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int g = per_sm * nsm;
  cache[key] = g;
  return g;
}

using LastInvTmaKernel = void (*)(const LastArgs<float>, unsigned);

template <int D, bool BATCH> LastInvTmaKernel last_inv_tma_kernel(int m) {
  switch (m) {
    case 16: return k_last_inv_tma<16, D, BATCH>;
    case 32: return k_last_inv_tma<32, D, BATCH>;
    case 64: return k_last_inv_tma<64, D, BATCH>;
    case 128: return k_last_inv_tma<128, D, BATCH>;
    case 256: return k_last_inv_tma<256, D, BATCH>;
    default: return nullptr;
  }
}

}  // namespace

// The staged rows need 16-byte aligned copies: an even row count (every tile, the
// last one included, holds an even number of rows of H complex values), an even
// number of k-points per plane and 16-byte aligned spectra (cudaMalloc'd; a batch's
// problems share the grid, so the host checks the first one).
int launch_last_inv_tma(Spectral &sp, const LastArgs<float> &a, int G, cudaStream_t s, int B) {
  const int dim = sp.g.dim, m = sp.ax[dim - 1].m, Y = reg_lanes(m), nc = sp.ncomp;
  if (nc != dim * dim || G % 2 || sp.g.nrows % 2 || sp.g.nk % 2 || (reinterpret_cast<uintptr_t>(sp.spec32) & 15))
    return 0;
  const bool batch = a.batch != nullptr;
  const LastInvTmaKernel k = dim == 2 ? (batch ? last_inv_tma_kernel<2, true>(m) : last_inv_tma_kernel<2, false>(m))
                                      : (batch ? last_inv_tma_kernel<3, true>(m) : last_inv_tma_kernel<3, false>(m));
  const int threads = Y * nc * (G / 2);
  const size_t smem = k_last_inv_tma_smem(m, nc, G);
  if (!k || threads > 224 || smem > (size_t)optin_smem()) return 0;  // launch bounds of the kernel
  allow_smem(k);
  const int per_grid = persistent_grid((const void *)k, threads, smem);
  if (per_grid < 1) return 0;
  const long long ntiles = (sp.g.nrows + G - 1) / G;
  const int grid = (int)std::min<long long>(ntiles, per_grid);
  launch_pdl(k, dim3(grid, B), dim3(Y, nc * (G / 2)), smem, s, a, (unsigned)last_inv_tma_stage(m, nc, G));
  MUSG_CHECK_LAUNCH();
  return grid;
}

// The descriptor is 5-D over the FP32 spectrum [comp][e][rho]: (rho, row group,
// component in the group, e div Y, e mod Y), box (Tt, 1, NC, R1, Y).  It needs a
// 16-byte aligned base, even row and plane counts (every stride a multiple of 16
// bytes) and an even tile width (every tile starts on a 16-byte boundary); tiles of 8
// or 16 pencils have kernels.
bool launch_green_tma(Spectral &sp, int mode, const GreenArgs<float> &a, int Tt, cudaStream_t s) {
  const int dim = sp.g.dim, m = sp.ax[0].m, Y = reg_lanes(m), R1 = RegLanesR1(m);
  const long long Rr = a.Rr, nk = sp.g.nk;
  if ((mode != GM_FINITE && mode != GM_SMALL) || Rr % 2 || nk % 2 ||
      (reinterpret_cast<uintptr_t>(sp.spec32) & 15))
    return false;
  const bool fin = mode == GM_FINITE;
  const int NC = fin ? dim : dim * dim, NG = fin ? dim : 1;
  GreenTmaKernel k = Tt == 8 ? green_tma_kernel<8>(mode, dim, m) : Tt == 16 ? green_tma_kernel<16>(mode, dim, m) : nullptr;
  const size_t smem = k_green_tma_smem(m, NC, Tt);
  if (!k || smem > (size_t)optin_smem() || Tt * Y * NC > 384) return false;
  if (sp.green_tmap_spec != sp.spec32 || sp.green_tmap_T != Tt || sp.green_tmap_mode != mode) {
    sp.green_tmap_spec = nullptr;
    EncodeTiledFn enc = encode_tiled_fn();
    if (!enc) return false;
    CUtensorMap map;
    const cuuint64_t e8 = sizeof(float2);
    const cuuint64_t gdim[5] = {(cuuint64_t)Rr, (cuuint64_t)NG, (cuuint64_t)NC, (cuuint64_t)R1, (cuuint64_t)Y};
    const cuuint64_t gstride[4] = {(cuuint64_t)nk * e8, (cuuint64_t)(fin ? dim : 1) * nk * e8,
                                   (cuuint64_t)Y * Rr * e8, (cuuint64_t)Rr * e8};
    const cuuint32_t box[5] = {(cuuint32_t)Tt, 1, (cuuint32_t)NC, (cuuint32_t)R1, (cuuint32_t)Y};
    const cuuint32_t estride[5] = {1, 1, 1, 1, 1};
    if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 5, sp.spec32, gdim, gstride, box, estride,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
    static_assert(sizeof(CUtensorMap) == sizeof(sp.green_tmap), "tensor map size");
    memcpy(sp.green_tmap, &map, sizeof(map));
    allow_smem(k);
    int per_sm = 0, dev = 0, nsm = 0;
    MUSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, Tt * Y * NC, smem));
    MUSG_CUDA(cudaGetDevice(&dev));
    MUSG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    if (per_sm < 1) return false;
    const long long ntiles = (Rr + Tt - 1) / Tt * NG;
    sp.green_tmap_grid = (int)std::min<long long>(ntiles, (long long)nsm * per_sm);
    sp.green_tmap_T = Tt;
    sp.green_tmap_mode = mode;
    sp.green_tmap_spec = sp.spec32;
  }
  CUtensorMap map;
  memcpy(&map, sp.green_tmap, sizeof(map));
  launch_pdl(k, dim3(sp.green_tmap_grid), dim3(Tt, Y, NC), smem, s, a, map);
  MUSG_CHECK_LAUNCH();
  return true;
}

}  // namespace musg
