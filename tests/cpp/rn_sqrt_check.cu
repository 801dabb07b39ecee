// Compares rn_sqrt and rn_sqrt2 (fluidsimulator_gb300/csrc/pbf_sqrt.cuh) with
// the IEEE square root, bit for bit, for every float in [kRnSqrtLo,
// kRnSqrtHi). Prints one JSON line; exits 0 when the comparison ran.
#include <cstdint>
#include <cstdio>

#include "pbf_sqrt.cuh"

using namespace fgb;

// neg_zero: -0.0f passed at run time, as the step passes SceneConst::neg_zero.
__global__ void check(uint32_t lo, uint32_t count, unsigned long long* bad, uint32_t* first, int paired,
                      float neg_zero) {
  const uint32_t stride = gridDim.x * blockDim.x;
  const float2 nz = make_float2(neg_zero, neg_zero);
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride) {
    const uint32_t bits = lo + k;
    const float x = __uint_as_float(bits);
    bool ok;
    if (paired) {
      // x in one half and its neighbour (bits ^ 1, inside the range too: lo
      // and hi are even) in the other, so each value is checked in both halves
      const float o = __uint_as_float(bits ^ 1u);
      const float2 r = rn_sqrt2(make_float2(x, o), nz);
      ok = __float_as_uint(r.x) == __float_as_uint(__fsqrt_rn(x)) &&
           __float_as_uint(r.y) == __float_as_uint(__fsqrt_rn(o));
    } else {
      ok = __float_as_uint(rn_sqrt(x)) == __float_as_uint(__fsqrt_rn(x));
    }
    if (!ok) {
      if (atomicAdd(bad, 1ull) == 0ull) *first = bits;
    }
  }
}

int main() {
  const uint32_t lo = __builtin_bit_cast(uint32_t, kRnSqrtLo);
  const uint32_t hi = __builtin_bit_cast(uint32_t, kRnSqrtHi);
  unsigned long long* bad = nullptr;
  uint32_t* first = nullptr;
  if (cudaMalloc(&bad, sizeof(*bad)) != cudaSuccess || cudaMalloc(&first, sizeof(*first)) != cudaSuccess) return 2;
  printf("{\"lo\": \"0x%08x\", \"hi\": \"0x%08x\", \"values\": %u", lo, hi, hi - lo);
  for (int paired = 0; paired < 2; ++paired) {
    cudaMemset(bad, 0, sizeof(*bad));
    cudaMemset(first, 0, sizeof(*first));
    check<<<152 * 8, 256>>>(lo, hi - lo, bad, first, paired, -0.0f);
    if (cudaDeviceSynchronize() != cudaSuccess) return 3;
    unsigned long long hb = 0;
    uint32_t hf = 0;
    cudaMemcpy(&hb, bad, sizeof(hb), cudaMemcpyDeviceToHost);
    cudaMemcpy(&hf, first, sizeof(hf), cudaMemcpyDeviceToHost);
    printf(", \"%s_mismatches\": %llu, \"%s_first\": \"0x%08x\"", paired ? "paired" : "scalar", hb,
           paired ? "paired" : "scalar", hf);
  }
  printf("}\n");
  return 0;
}
