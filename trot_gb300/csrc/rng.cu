// Device-side auxiliary-field sampling.
//
// The reference draws the fields of every step with jax.random.normal from a
// key it splits each step (trot/prop/afqmc.py:91-93) and the SR zeta with
// jax.random.uniform (trot/prop/blocks.py:270-271).  Here the key is two
// uint32 words kept on the device (stored in int64 slots), and numbers come
// from the counter-based Philox-4x32-10 generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), so sampling needs no
// host round trip and can sit inside a captured CUDA graph.
//   split:   key' = philox((0, 0, 0, 1), key)[0:2],  sub = philox((0, 0, 0, 2), key)[0:2]
//   normals: for walker b, pair j: philox((j, b, 0x5eed, 0), sub) -> 4 words ->
//            two 53-bit uniforms u1, u2 in (0, 1) -> Box-Muller
//            z(b, 2j) = sqrt(-2 log u1) cos(2 pi u2), z(b, 2j+1) = ... sin(2 pi u2)
//   uniform: philox((k, 0, 0x2e7a, 0), sub) -> one 53-bit uniform in [0, 1)
#include "kernels.h"

namespace trot {

struct U4 { uint32_t x, y, z, w; };

TROT_HD U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)M0 * c.x, p1 = (uint64_t)M1 * c.z;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// 53-bit uniform strictly inside (0, 1) from two words
TROT_HD double uniform_open(uint32_t a, uint32_t b) {
  const uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return ((double)m + 0.5) * (1.0 / 9007199254740992.0);
}
// 53-bit uniform in [0, 1)
TROT_HD double uniform_closed_open(uint32_t a, uint32_t b) {
  const uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return (double)m * (1.0 / 9007199254740992.0);
}

TROT_D void subkey(const long long* key, uint32_t& s0, uint32_t& s1) {
  const U4 r = philox4x32_10(U4{0, 0, 0, 2}, (uint32_t)key[0], (uint32_t)key[1]);
  s0 = r.x;
  s1 = r.y;
}

__global__ void normal_fields_kernel(const long long* __restrict__ key, int W, int G, double* __restrict__ out) {
  uint32_t s0, s1;
  subkey(key, s0, s1);
  const int npair = (G + 1) / 2;
  const long long total = (long long)W * npair;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(t / npair), j = (int)(t % npair);
    const U4 r = philox4x32_10(U4{(uint32_t)j, (uint32_t)b, 0x5eedu, 0u}, s0, s1);
    const double u1 = uniform_open(r.x, r.y), u2 = uniform_open(r.z, r.w);
    const double rad = sqrt(-2.0 * log(u1));
    double sn, cs;
    sincospi(2.0 * u2, &sn, &cs);
    double* o = out + (size_t)b * G + 2 * j;
    o[0] = rad * cs;
    if (2 * j + 1 < G) o[1] = rad * sn;
  }
}

__global__ void uniform_kernel(const long long* __restrict__ key, int n, double* __restrict__ out) {
  uint32_t s0, s1;
  subkey(key, s0, s1);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const U4 r = philox4x32_10(U4{(uint32_t)k, 0u, 0x2e7au, 0u}, s0, s1);
    out[k] = uniform_closed_open(r.x, r.y);
  }
}

__global__ void split_key_kernel(long long* key) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const U4 r = philox4x32_10(U4{0, 0, 0, 1}, (uint32_t)key[0], (uint32_t)key[1]);
    key[0] = (long long)r.x;
    key[1] = (long long)r.y;
  }
}

}  // namespace trot

using namespace trot;

extern "C" {

int trot_sample_normal_fields(const int64_t* key, int n_walkers, int nchol, double* fields, void* stream) {
  if (!key || !fields) { set_error("null key or fields"); return TROT_ERR_NULL_PTR; }
  if (n_walkers <= 0 || nchol <= 0) { set_error("bad sizes"); return TROT_ERR_BAD_SHAPE; }
  long long total = (long long)n_walkers * ((nchol + 1) / 2);
  int grid = (int)((total + 255) / 256);
  if (grid > 152 * 16) grid = 152 * 16;
  normal_fields_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>((const long long*)key, n_walkers, nchol, fields);
  TROT_CHECK_LAUNCH("normal_fields_kernel");
  return TROT_OK;
}

int trot_sample_uniform(const int64_t* key, int n, double* out, void* stream) {
  if (!key || !out) { set_error("null key or output"); return TROT_ERR_NULL_PTR; }
  if (n <= 0) { set_error("bad size"); return TROT_ERR_BAD_SHAPE; }
  uniform_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>((const long long*)key, n, out);
  TROT_CHECK_LAUNCH("uniform_kernel");
  return TROT_OK;
}

int trot_split_key(int64_t* key, void* stream) {
  if (!key) { set_error("null key"); return TROT_ERR_NULL_PTR; }
  split_key_kernel<<<1, 32, 0, (cudaStream_t)stream>>>((long long*)key);
  TROT_CHECK_LAUNCH("split_key_kernel");
  return TROT_OK;
}

}  // extern "C"
