// Plain BF16 tcgen05 GEMM, D (M x N, f32) = A (M x K, bf16) * B (N x K, bf16)^T,
// all row-major / K-major.  It is the tested building block of the tensor-core
// kernels (same descriptors, TMEM handling and bounded waits) and a usable
// library GEMM for 128-aligned shapes.
#include "kernels.h"
#include "tc.cuh"

namespace trot {

static constexpr int kTcBM = 128, kTcBN = 128, kTcBK = 64;

__global__ void __launch_bounds__(128)
tc_gemm_bf16_kernel(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B, float* __restrict__ D, int M,
                    int N, int K, int* __restrict__ status) {
  __shared__ __align__(1024) unsigned char sA[kTcBM * kTcBK * 2];
  __shared__ __align__(1024) unsigned char sB[kTcBN * kTcBK * 2];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * kTcBM, n0 = blockIdx.x * kTcBN;
  if (warp == 0) tc::tmem_alloc(&tslot, kTcBN);
  if (tid == 0) tc::mbar_init(&mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = tslot;
  const uint32_t idesc = tc::idesc_bf16_f32(kTcBM, kTcBN);
  const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
  bool ok = true;
  const int nk = K / kTcBK;
  for (int kt = 0; kt < nk && ok; ++kt) {
    const int k0 = kt * kTcBK;
    // 16-byte chunks: (row r, k group g) -> core-matrix layout
    for (int c = tid; c < kTcBM * 8; c += 128) {
      const int r = c >> 3, g = c & 7;
      *reinterpret_cast<uint4*>(sA + tc::tile_off(r, g * 8)) =
          *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * K + k0 + g * 8);
    }
    for (int c = tid; c < kTcBN * 8; c += 128) {
      const int r = c >> 3, g = c & 7;
      *reinterpret_cast<uint4*>(sB + tc::tile_off(r, g * 8)) =
          *reinterpret_cast<const uint4*>(B + (size_t)(n0 + r) * K + k0 + g * 8);
    }
    tc::fence_proxy_async();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
#pragma unroll
      for (int ks = 0; ks < kTcBK / 16; ++ks) {
        const uint64_t ad = tc::smem_desc(a0 + ks * 256, 128, 1024);
        const uint64_t bd = tc::smem_desc(b0 + ks * 256, 128, 1024);
        tc::mma_bf16(taddr, ad, bd, idesc, (kt > 0 || ks > 0) ? 1u : 0u);
      }
      tc::mma_commit(&mbar);
    }
    ok = tc::mbar_wait(&mbar, kt & 1);
    __syncthreads();
  }
  if (!ok) {
    if (tid == 0) atomicExch(status, (int)TROT_ERR_DEVICE_TIMEOUT);
  } else {
    tc::fence_after_sync();
    const uint32_t trow = taddr + ((uint32_t)(warp * 32) << 16);
    float v[16];
    for (int c = 0; c < kTcBN / 16; ++c) {
      tc::tmem_ld16(trow + c * 16, v);
      float* d = D + (size_t)(m0 + warp * 32 + lane) * N + n0 + c * 16;
#pragma unroll
      for (int i = 0; i < 16; ++i) d[i] = v[i];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, kTcBN);
}

}  // namespace trot

extern "C" int trot_tc_gemm_bf16(const uint16_t* A, const uint16_t* B, float* D, int M, int N, int K,
                                 int* status, void* stream) {
  using namespace trot;
  if (!A || !B || !D || !status) { set_error("null pointer"); return TROT_ERR_NULL_PTR; }
  if (M <= 0 || N <= 0 || K <= 0 || M % kTcBM || N % kTcBN || K % kTcBK) {
    set_error("tc_gemm_bf16: M, N must be multiples of 128 and K of 64 (got %d, %d, %d)", M, N, K);
    return TROT_ERR_BAD_SHAPE;
  }
  if (((uintptr_t)A | (uintptr_t)B) & 15) { set_error("tc_gemm_bf16: A, B must be 16-byte aligned"); return TROT_ERR_BAD_SHAPE; }
  dim3 grid(N / kTcBN, M / kTcBM);
  tc_gemm_bf16_kernel<<<grid, 128, 0, (cudaStream_t)stream>>>(A, B, D, M, N, K, status);
  TROT_CHECK_LAUNCH("tc_gemm_bf16_kernel");
  return TROT_OK;
}
