// Throughput of the warp-level (legacy) tensor-core instructions on this GPU,
// for the record of the tensor path the Ozaki qgemm uses: tcgen05.mma of
// kind::i8 (exact int8 -> int32) does not assemble for sm_103a, so the
// choice was between mma.sync int8 (exact int32 sums, the numerics of an
// int8 Ozaki split) and integer-valued fp16 digits on tcgen05.mma kind::f16.
//
// Each warp runs 8 independent accumulator chains of one instruction shape,
// ITERS steps each, in a grid of (SMs x 8) blocks of 4 warps; the rate is
// 2 * M * N * K * instructions / time (CUDA events around the launch, after
// a warm-up launch).  Prints one JSON line; exits nonzero on a CUDA error.
//   mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32   (int8, int32 accumulate)
//   mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 (fp16, fp32 accumulate)
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

constexpr int kIters = 4096;
constexpr int kChains = 8;

__global__ void __launch_bounds__(128) mma_s8_loop(int* out, int seed) {
  uint32_t a[4], b[2];
  for (int i = 0; i < 4; ++i) a[i] = 0x01010101u * (uint32_t)((threadIdx.x + i + seed) & 3);
  for (int i = 0; i < 2; ++i) b[i] = 0x01010101u * (uint32_t)((threadIdx.x * 3 + i) & 3);
  int d[kChains][4] = {};
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c)
      asm volatile(
          "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
          "{%0, %1, %2, %3};"
          : "+r"(d[c][0]), "+r"(d[c][1]), "+r"(d[c][2]), "+r"(d[c][3])
          : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
  }
  int s = 0;
  for (int c = 0; c < kChains; ++c) s += d[c][0] + d[c][1] + d[c][2] + d[c][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(128) mma_f16_loop(float* out, int seed) {
  uint32_t a[4], b[2];
  for (int i = 0; i < 4; ++i) a[i] = 0x3C003C00u * (uint32_t)(((threadIdx.x + i + seed) & 1));
  for (int i = 0; i < 2; ++i) b[i] = 0x3C003C00u * (uint32_t)(((threadIdx.x + i) & 1));
  float d[kChains][4] = {};
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c)
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
          "{%0, %1, %2, %3};"
          : "+f"(d[c][0]), "+f"(d[c][1]), "+f"(d[c][2]), "+f"(d[c][3])
          : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
  }
  float s = 0;
  for (int c = 0; c < kChains; ++c) s += d[c][0] + d[c][1] + d[c][2] + d[c][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename F>
static float time_ms(F launch) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch();  // warm-up
  cudaEventRecord(e0);
  launch();
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

int main() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 128;
  void* buf = nullptr;
  if (cudaMalloc(&buf, (size_t)blocks * threads * 4) != cudaSuccess) return 2;
  const double instr = (double)blocks * (threads / 32) * kChains * kIters;
  const float ms_s8 = time_ms([&] { mma_s8_loop<<<blocks, threads>>>((int*)buf, 1); });
  const float ms_f16 = time_ms([&] { mma_f16_loop<<<blocks, threads>>>((float*)buf, 1); });
  cudaError_t e = cudaDeviceSynchronize();
  cudaFree(buf);
  if (e != cudaSuccess) {
    fprintf(stderr, "CUDA error: %s\n", cudaGetErrorString(e));
    return 1;
  }
  const double s8 = 2.0 * 16 * 8 * 32 * instr / (ms_s8 * 1e-3) / 1e12;
  const double f16 = 2.0 * 16 * 8 * 16 * instr / (ms_f16 * 1e-3) / 1e12;
  printf("{\"sms\": %d, \"mma_sync_s8_tops\": %.1f, \"mma_sync_f16_tflops\": %.1f, \"ms_s8\": %.3f, "
         "\"ms_f16\": %.3f}\n",
         sms, s8, f16, ms_s8, ms_f16);
  return 0;
}
