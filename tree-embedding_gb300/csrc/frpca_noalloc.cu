// tsvd_frpca_noalloc: tsvd_frpca without any allocation.
//
// For callers that cannot allocate device memory: plug-ins living inside a
// host application that reserves the whole device memory pool for itself
// (its own allocator hands out every byte, so a cudaMalloc of ours fails or
// steals from it), and latency-bound host loops that must not go through the
// allocator (cudaMalloc and cudaFree can synchronize the device and stall the
// caller's other streams). Every buffer the randomized SVD needs lives in one
// file-scope __device__ array (g_noalloc_scratch, kNoallocScratchBytes bytes,
// held by every GPU that loads this library until the process exits), and
// every host-side staging buffer is a file-scope array as well. Inputs and
// outputs are the caller's, exactly as for tsvd_frpca.
//
// The call is synchronous: it runs on the legacy default stream (stream 0,
// so it is ordered with the caller's blocking streams), reads the count of
// non-empty columns back to the host midway, and returns once the results
// are in the caller's buffers.
//
// Limits (larger inputs are rejected with TSVD_ERR_INVALID before any GPU
// work): nrows <= 512, ncols <= 16384, at most 2048 non-empty columns,
// nnz <= 262144, k <= 64 (q is free), |values| <= FLT_MAX.
//
// Set-up: the first call on a device, with that device current, resolves the
// array's device address once (cudaGetSymbolAddress) and checks that the
// regions reserved for the Gram and Jacobi work areas hold what the kernels
// ask for at the limits; make that first call before any stream capture.
// Calls share the array: two calls that overlap on the GPU (from several host
// threads, or on several streams) race.
#include <cfloat>
#include <cmath>
#include <cstring>

#include "factor.h"
#include "internal.h"

using namespace tsvd;

namespace {

constexpr int kNaMaxRows = 512;
constexpr int kNaMaxCols = 16384;
constexpr int kNaMaxUsedCols = 2048;
constexpr int64_t kNaMaxNnz = 262144;
constexpr int kNaMaxK = 64;
constexpr int kNaMaxL = kNaMaxK + 5;

constexpr size_t al(size_t x) { return (x + 255) / 256 * 256; }

// Device scratch layout (byte offsets, each region 256-byte aligned).
constexpr size_t kAtB = al((size_t)kNaMaxUsedCols * kNaMaxRows * 2);
constexpr size_t kXB = al((size_t)kNaMaxUsedCols * kLp * 2);
constexpr size_t kZB = al(std::max((size_t)kNaMaxUsedCols * kLp, (size_t)kNaMaxRows * 256) * 4);
constexpr size_t kYB = al((size_t)kNaMaxRows * kLp * 4);
constexpr size_t kQB = al((size_t)kNaMaxRows * kLp * 2);
constexpr size_t kGB = al((size_t)256 * 256 * 8);
constexpr size_t kTB = al((size_t)kLp * kLp * 4);
constexpr size_t kLamB = al(256 * 4);
constexpr size_t kVB = al((size_t)256 * 256 * 4);
constexpr size_t kCsB = al(512 * 4);
constexpr size_t kSumB = al(8);
constexpr int64_t kGramChunks = (std::max(kNaMaxUsedCols, kNaMaxRows) + 127) / 128 + 1;
constexpr size_t kGramB = al((size_t)kGramChunks * kNaMaxL * kNaMaxL * 8);
constexpr size_t kJacB = al((size_t)30 * (kNaMaxL + 1) * ((kNaMaxL + 1) / 2) * 8) + 512 + al(kNaMaxL * 4);
constexpr size_t kPtrSlots = 320;
constexpr size_t kPtrB = al(kPtrSlots * 8);
constexpr size_t kIntB = al(kPtrSlots * 4);
constexpr size_t kRowPtrB = al((size_t)(kNaMaxRows + 1) * 8);
constexpr size_t kColB = al((size_t)kNaMaxNnz * 4);
constexpr size_t kValB = al((size_t)kNaMaxNnz * 8);
constexpr size_t kCinvB = al((size_t)kNaMaxCols * 4);
constexpr size_t kCmapB = al((size_t)kNaMaxUsedCols * 4);
constexpr size_t kUB = al((size_t)kNaMaxRows * kNaMaxK * 4);
constexpr size_t kVoutB = al((size_t)kNaMaxUsedCols * kNaMaxK * 4);
constexpr size_t kSigB = al(kNaMaxK * 4);
constexpr size_t kMiscB = al(16);
constexpr size_t kRefB = al((size_t)kNaMaxL * kNaMaxL * 8);  // eigen refinement (fp64)
constexpr size_t kHpB = al(8);                                // device pointer to dh
constexpr size_t kTmapB = al(6 * sizeof(CUtensorMap));        // the products' tensor maps

constexpr size_t kOffAt = 0;
constexpr size_t kOffXhi = kOffAt + kAtB;
constexpr size_t kOffXlo = kOffXhi + kXB;
constexpr size_t kOffZ = kOffXlo + kXB;
constexpr size_t kOffY = kOffZ + kZB;
constexpr size_t kOffQhi = kOffY + kYB;
constexpr size_t kOffQlo = kOffQhi + kQB;
constexpr size_t kOffG = kOffQlo + kQB;
constexpr size_t kOffT = kOffG + kGB;
constexpr size_t kOffLam = kOffT + kTB;
constexpr size_t kOffV = kOffLam + kLamB;
constexpr size_t kOffCs = kOffV + kVB;
constexpr size_t kOffSum = kOffCs + kCsB;
constexpr size_t kOffGram = kOffSum + kSumB;
constexpr size_t kOffJac = kOffGram + kGramB;
constexpr size_t kOffPtr = kOffJac + kJacB;
constexpr size_t kOffInt = kOffPtr + kPtrB;
constexpr size_t kOffRowPtr = kOffInt + kIntB;
constexpr size_t kOffCol = kOffRowPtr + kRowPtrB;
constexpr size_t kOffVal = kOffCol + kColB;
constexpr size_t kOffCinv = kOffVal + kValB;
constexpr size_t kOffCmap = kOffCinv + kCinvB;
constexpr size_t kOffU = kOffCmap + kCmapB;
constexpr size_t kOffVout = kOffU + kUB;
constexpr size_t kOffSig = kOffVout + kVoutB;
constexpr size_t kOffMisc = kOffSig + kSigB;
constexpr size_t kOffDv = kOffMisc + kMiscB;
constexpr size_t kOffDt = kOffDv + kRefB;
constexpr size_t kOffDh = kOffDt + kRefB;
constexpr size_t kOffHp = kOffDh + kRefB;
constexpr size_t kOffTmap = kOffHp + kHpB;
constexpr size_t kNoallocScratchBytes = kOffTmap + kTmapB;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Host staging (pointer arrays, results), also static.
void *g_hptr[kPtrSlots];
int32_t g_hint[kPtrSlots];
float g_hu[kNaMaxRows * kNaMaxK];
float g_hv[kNaMaxUsedCols * kNaMaxK];
float g_hs[kNaMaxK];
int32_t g_hcmap[kNaMaxUsedCols];
alignas(64) CUtensorMap g_htmap[6];

constexpr int kMaxDevices = 64;
unsigned char *g_dev_scratch[kMaxDevices] = {nullptr};

// misc: [0..1] max |value| as the bits of a double (non-negative doubles
// order like their bit patterns, so an integer maximum finds the largest
// magnitude exactly as tsvd_frpca's host loop does), [2] non-empty columns
__global__ void na_mark_kernel(const int64_t *row_ptr, const int32_t *col, const double *val,
                               int nrows, int32_t *cinv, uint32_t *misc) {
  unsigned long long *vmax_bits = reinterpret_cast<unsigned long long *>(misc);
  for (int i = blockIdx.x; i < nrows; i += gridDim.x)
    for (int64_t t = row_ptr[i] + threadIdx.x; t < row_ptr[i + 1]; t += blockDim.x) {
      double v = val[t];
      if (v == 0.0) continue;
      cinv[col[t]] = 1;
      atomicMax(vmax_bits, (unsigned long long)__double_as_longlong(fabs(v)));
    }
}

__global__ void na_rebase_kernel(int64_t *row_ptr, int nrows, int32_t *col, int64_t nnz) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= nrows || i < nnz;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i <= nrows) row_ptr[i] -= 1;
    if (i < nnz) col[i] -= 1;
  }
}

// One CTA: exclusive scan of the column flags into compacted indices.
__global__ void na_compact_kernel(int32_t *cinv, int ncols, int32_t *cmap, uint32_t *misc) {
  __shared__ int32_t base;
  __shared__ int32_t wsum[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  for (int c0 = 0; c0 < ncols; c0 += blockDim.x) {
    int c = c0 + threadIdx.x;
    int f = c < ncols && cinv[c] == 1;
    unsigned m = __ballot_sync(0xffffffffu, f);
    if (lane == 0) wsum[warp] = __popc(m);
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      if (w < warp) before += wsum[w];
      total += wsum[w];
    }
    if (c < ncols) {
      if (f) {
        int idx = base + before + __popc(m & ((1u << lane) - 1u));
        cinv[c] = idx;
        if (idx < kNaMaxUsedCols) cmap[idx] = c;
      } else {
        cinv[c] = -1;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) base += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) misc[2] = (uint32_t)base;
}

__global__ void na_densify_kernel(const int64_t *row_ptr, const int32_t *col, const double *val,
                                  int nrows, const int32_t *cinv, int sp, float scale,
                                  __half *at) {
  for (int i = blockIdx.x; i < nrows; i += gridDim.x)
    for (int64_t t = row_ptr[i] + threadIdx.x; t < row_ptr[i + 1]; t += blockDim.x) {
      double v = val[t];
      int c = cinv[col[t]];
      if (v == 0.0 || c < 0) continue;
      at[(int64_t)c * sp + i] = __float2half_rn((float)(v * scale));
    }
}

tsvd_status scratch_for_current_device(unsigned char **out) {
  int dev = 0;
  TSVD_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(TSVD_ERR_INVALID, "device %d", dev);
  if (!g_dev_scratch[dev]) {
    // the fixed regions must hold what the shared kernels ask for at the limits
    const size_t gram_need = gram_work_bytes(std::max(kNaMaxUsedCols, kNaMaxRows), kNaMaxL, 1);
    const size_t jac_need = jacobi_work_bytes(kNaMaxL, 1);
    if (gram_need > kGramB || jac_need > kJacB)
      return fail(TSVD_ERR_STATE,
                  "frpca_noalloc: static scratch too small for the kernels (Gram %zu > %zu or "
                  "Jacobi %zu > %zu bytes)", gram_need, kGramB, jac_need, kJacB);
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(TSVD_ERR_DEVICE, "cudaGetSymbolAddress(g_noalloc_scratch): %s",
                  cudaGetErrorString(e));
    g_dev_scratch[dev] = (unsigned char *)p;
  }
  *out = g_dev_scratch[dev];
  return TSVD_OK;
}

}  // namespace

extern "C" tsvd_status tsvd_frpca_noalloc(int32_t nrows, int32_t ncols, int64_t nnz,
                                          const int64_t *row_ptr, const int32_t *col_idx,
                                          const double *values, int32_t index_base, int32_t k,
                                          int32_t q, uint64_t seed, double *U, double *S,
                                          double *V) {
  if (nrows < 1 || ncols < 1 || nnz < 0 || !row_ptr || (nnz > 0 && (!col_idx || !values)))
    return fail(TSVD_ERR_INVALID, "frpca_noalloc: bad matrix arguments");
  if (nrows > kNaMaxRows || ncols > kNaMaxCols || nnz > kNaMaxNnz || k < 1 || k > kNaMaxK ||
      q < 1)
    return fail(TSVD_ERR_INVALID,
                "frpca_noalloc: limits are nrows <= %d, ncols <= %d, nnz <= %lld, 1 <= k <= %d, "
                "q >= 1 (got %d, %d, %lld, %d, %d)",
                kNaMaxRows, kNaMaxCols, (long long)kNaMaxNnz, kNaMaxK, nrows, ncols,
                (long long)nnz, k, q);
  if (index_base != 0 && index_base != 1)
    return fail(TSVD_ERR_INVALID, "frpca_noalloc: index_base");
  if (row_ptr[0] != index_base || row_ptr[nrows] - index_base != nnz)
    return fail(TSVD_ERR_INVALID, "frpca_noalloc: row pointers do not span nnz");
  for (int32_t i = 0; i < nrows; ++i)
    if (row_ptr[i + 1] < row_ptr[i]) return fail(TSVD_ERR_INVALID, "frpca_noalloc: row pointers");
  for (int64_t t = 0; t < nnz; ++t) {
    int32_t c = col_idx[t] - index_base;
    if (c < 0 || c >= ncols) return fail(TSVD_ERR_INVALID, "frpca_noalloc: column out of range");
    if (!std::isfinite(values[t])) return fail(TSVD_ERR_NUMERIC, "frpca_noalloc: non-finite value");
    if (std::fabs(values[t]) > (double)FLT_MAX)
      return fail(TSVD_ERR_INVALID, "frpca_noalloc: |value| above the float range");
  }
  unsigned char *base = nullptr;
  TSVD_TRY(scratch_for_current_device(&base));
  cudaStream_t st = 0;
  const int sp = (int)round_up(nrows, kRowPad);
  const int l = k + 5;
  // CSR into the array; indices are rebased to 0 on the device side copy
  int64_t *d_rp = (int64_t *)(base + kOffRowPtr);
  int32_t *d_col = (int32_t *)(base + kOffCol);
  double *d_val = (double *)(base + kOffVal);
  int32_t *d_cinv = (int32_t *)(base + kOffCinv);
  int32_t *d_cmap = (int32_t *)(base + kOffCmap);
  uint32_t *d_misc = (uint32_t *)(base + kOffMisc);
  TSVD_CUDA(cudaMemcpyAsync(d_rp, row_ptr, sizeof(int64_t) * (nrows + 1), cudaMemcpyHostToDevice, st));
  if (nnz > 0) {
    TSVD_CUDA(cudaMemcpyAsync(d_col, col_idx, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, st));
    TSVD_CUDA(cudaMemcpyAsync(d_val, values, sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
  }
  // the array keeps the previous call's contents: clear what must start at 0
  TSVD_CUDA(cudaMemsetAsync(d_cinv, 0, sizeof(int32_t) * ncols, st));
  TSVD_CUDA(cudaMemsetAsync(d_misc, 0, kMiscB, st));
  {
    // the fp64 refinement reads its matrix through a one-entry pointer array
    // in the scratch: written on every call, so the array never relies on
    // what an earlier call (or an earlier context) left there
    static double *dh_host[kMaxDevices];
    int dev = 0;
    TSVD_CUDA(cudaGetDevice(&dev));
    dh_host[dev] = (double *)(base + kOffDh);
    TSVD_CUDA(cudaMemcpyAsync(base + kOffHp, &dh_host[dev], sizeof(double *),
                              cudaMemcpyHostToDevice, st));
  }
  TSVD_CUDA(cudaMemsetAsync(base + kOffAt, 0, kAtB, st));
  const int grid = std::min(nrows, 4 * sm_count());
  if (index_base == 1) {  // rebase the copied indices to 0
    na_rebase_kernel<<<grid, 256, 0, st>>>(d_rp, nrows, d_col, nnz);
    TSVD_LAUNCH_CHECK();
  }
  na_mark_kernel<<<grid, 128, 0, st>>>(d_rp, d_col, d_val, nrows, d_cinv, d_misc);
  TSVD_LAUNCH_CHECK();
  na_compact_kernel<<<1, 1024, 0, st>>>(d_cinv, ncols, d_cmap, d_misc);
  TSVD_LAUNCH_CHECK();
  uint32_t hmisc[4];
  TSVD_CUDA(cudaMemcpyAsync(hmisc, d_misc, sizeof hmisc, cudaMemcpyDeviceToHost, st));
  TSVD_CUDA(cudaStreamSynchronize(st));
  const int32_t nc = (int32_t)hmisc[2];
  if (nc > kNaMaxUsedCols)
    return fail(TSVD_ERR_INVALID, "frpca_noalloc: %d non-empty columns > %d", nc, kNaMaxUsedCols);
  double vmax;
  std::memcpy(&vmax, &hmisc[0], sizeof vmax);
  int e2 = 0;
  if (vmax > 0) std::frexp(vmax, &e2);
  const double scale = std::ldexp(1.0, 14 - e2);
  if (nc > 0) {
    na_densify_kernel<<<grid, 128, 0, st>>>(d_rp, d_col, d_val, nrows, d_cinv, sp, (float)scale,
                                            (__half *)(base + kOffAt));
    TSVD_LAUNCH_CHECK();
    FrpcaWork W;
    W.nmax = 1;
    W.rows_max = kNaMaxUsedCols;
    W.sp = sp;
    W.l = l;
    W.d = k;
    W.xhi = (__half *)(base + kOffXhi);
    W.xlo = (__half *)(base + kOffXlo);
    W.z = (float *)(base + kOffZ);
    W.y = (float *)(base + kOffY);
    W.qhi = (__half *)(base + kOffQhi);
    W.qlo = (__half *)(base + kOffQlo);
    W.g = (double *)(base + kOffG);
    W.t = (float *)(base + kOffT);
    W.lambda = (float *)(base + kOffLam);
    W.v = (float *)(base + kOffV);
    W.colscale = (float *)(base + kOffCs);
    W.sums = (double *)(base + kOffSum);
    W.gram_work = (double *)(base + kOffGram);
    W.gram_bytes = kGramB;
    W.jac_work = base + kOffJac;
    W.jac_bytes = kJacB;
    W.dptr = (void **)(base + kOffPtr);
    W.hptr = g_hptr;
    W.ptr_slots = kPtrSlots;
    W.dint = (int32_t *)(base + kOffInt);
    W.hint = g_hint;
    W.dv = (double *)(base + kOffDv);
    W.dt = (double *)(base + kOffDt);
    W.dh = (double *)(base + kOffDh);
    W.dh_ptrs = (double **)(base + kOffHp);
    W.tmap_dev = (CUtensorMap *)(base + kOffTmap);
    W.tmap_host = g_htmap;
    W.tmap_slots = 6;
    FrpcaProblem P;
    P.block = 0;
    P.at = (const __half *)(base + kOffAt);
    P.ncols = nc;
    P.colmap = d_cmap;
    P.col_base = 0;
    P.b_out = nullptr;
    P.sigma_out = (float *)(base + kOffSig);
    P.u_out = (float *)(base + kOffU);
    P.v_out = (float *)(base + kOffVout);
    double ssum = 0.0;
    TSVD_TRY(frpca_batch(W, &P, 1, q, seed, nrows, st, &ssum));
    TSVD_CUDA(cudaMemcpyAsync(g_hu, P.u_out, sizeof(float) * nrows * k, cudaMemcpyDeviceToHost, st));
    TSVD_CUDA(cudaMemcpyAsync(g_hv, P.v_out, sizeof(float) * nc * k, cudaMemcpyDeviceToHost, st));
    TSVD_CUDA(cudaMemcpyAsync(g_hs, P.sigma_out, sizeof(float) * k, cudaMemcpyDeviceToHost, st));
    TSVD_CUDA(cudaMemcpyAsync(g_hcmap, d_cmap, sizeof(int32_t) * nc, cudaMemcpyDeviceToHost, st));
    TSVD_CUDA(cudaStreamSynchronize(st));
  }
  for (int j = 0; j < k; ++j) {
    if (S) S[j] = nc > 0 ? g_hs[j] / scale : 0.0;
    if (U)
      for (int32_t i = 0; i < nrows; ++i)
        U[(size_t)j * nrows + i] = nc > 0 ? g_hu[(size_t)i * k + j] : 0.0;
    if (V) {
      for (int32_t c = 0; c < ncols; ++c) V[(size_t)j * ncols + c] = 0.0;
      for (int32_t c = 0; c < nc; ++c) V[(size_t)j * ncols + g_hcmap[c]] = g_hv[(size_t)c * k + j];
    }
  }
  return TSVD_OK;
}
