/*
 * FP64 pipe throughput probe, used by bench.py as the denominator of the FP64
 * roofline (the measured-peaks file has HBM and bf16 figures only).  Eight
 * independent add/multiply chains per thread, 16 warps per SM, timed with CUDA
 * events; reports binary64 add/multiply lane-operations per second.
 */
#include <cuda_runtime.h>

__global__ void k_fp64_chains(double* out, int iters) {
  double a0 = threadIdx.x * 1e-3 + 1.0, a1 = a0 + 0.1, a2 = a0 + 0.2, a3 = a0 + 0.3;
  double a4 = a0 + 0.4, a5 = a0 + 0.5, a6 = a0 + 0.6, a7 = a0 + 0.7;
  const double b = 1.0000001, c = 0.9999999;
  for (int i = 0; i < iters; ++i) {
    a0 = __dadd_rn(a0, b); a1 = __dmul_rn(a1, c); a2 = __dadd_rn(a2, c); a3 = __dmul_rn(a3, b);
    a4 = __dadd_rn(a4, b); a5 = __dmul_rn(a5, c); a6 = __dadd_rn(a6, c); a7 = __dmul_rn(a7, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

extern "C" int shapes_probe_fp64(double* lane_ops_per_s) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -5;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -5;
  const int threads = 256, blocks = sms * 2, iters = 20000;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * threads * blocks) != cudaSuccess) return -5;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_chains<<<blocks, threads>>>(d, 64);
  cudaEventRecord(e0);
  k_fp64_chains<<<blocks, threads>>>(d, iters);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (err != cudaSuccess || ms <= 0.f) return -5;
  *lane_ops_per_s = (double)blocks * threads * iters * 8.0 / (ms * 1e-3);
  return 0;
}

/*
 * Self-checks of the exact binary64 helpers (fp64_ops.cuh) against the
 * hardware IEEE operations they replace; used by the test suite.
 */
#include "fp64_ops.cuh"

namespace {

__host__ __device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  /* splitmix64 finaliser (Steele, Lea, Flood 2014) */
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ double make_double(unsigned long long sign, int exp, unsigned long long mant) {
  return __longlong_as_double((long long)((sign << 63) | ((unsigned long long)exp << 52) | (mant & 0xfffffffffffffull)));
}

/* Operand classes: random mantissas over the whole fast range and beyond it,
 * all-ones and all-zeros mantissas, mantissas of the form 2^k +- 1, and
 * numerators built as b * q with short-mantissa q (quotients near exact). */
__device__ void div_operands(unsigned long long k, unsigned long long seed, double* a, double* b) {
  const unsigned long long r0 = mix64(k ^ seed), r1 = mix64(r0), r2 = mix64(r1), r3 = mix64(r2);
  const int cls = (int)(r3 % 6);
  const int eb = 523 + (int)(r1 % 1000);   /* recip_ok range */
  int ea = 600 + (int)(r2 % 850);          /* straddles the fast range */
  unsigned long long mb = r0, ma = r2 >> 3;
  if (cls == 1) mb = 0xfffffffffffffull;
  if (cls == 2) mb = 0;
  if (cls == 3) mb = (1ull << (r1 % 52)) + ((r0 & 1) ? 1ull : 0xfffffffffffffull);
  if (cls == 4) ma = 0xfffffffffffffull;
  *b = make_double(r1 >> 63, eb, mb);
  if (cls == 5) {
    const double q = make_double(r2 >> 63, 1023 + (int)(r0 % 64) - 32, (r1 >> 12) & 0xfff0000000000ull);
    *a = *b * q;
  } else {
    *a = make_double(r0 >> 63, ea, ma);
  }
}

__global__ void k_div_check(unsigned long long n, unsigned long long seed, unsigned long long* bad,
                            double* first) {
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    double a, b;
    div_operands(k, seed, &a, &b);
    const double y = shapes::recip_ok(b) ? 1.0 / b : 0.0;
    const double q = shapes::div_rn(a, b, y);
    const double ref = a / b;
    if (__double_as_longlong(q) != __double_as_longlong(ref)) {
      if (atomicAdd(bad, 1ull) == 0) {
        first[0] = a;
        first[1] = b;
      }
    }
  }
}

/* Operand classes for mul_rn_int: random mantissas with exponents straddling
 * the fast range, short (sparse) mantissas whose products are exact or exact
 * ties, all-ones / 2^k +- 1 mantissas, products next to overflow, zeros next
 * to finite and non-finite values, and subnormal, infinite and NaN operands. */
__device__ void mul_operands(unsigned long long k, unsigned long long seed, double* a, double* b) {
  const unsigned long long r0 = mix64(k ^ seed), r1 = mix64(r0), r2 = mix64(r1), r3 = mix64(r2);
  const int cls = (int)(r3 % 8);
  int ea = 480 + (int)(r1 % 1091), eb = 480 + (int)(r2 % 1091); /* [480, 1570] */
  unsigned long long ma = r0, mb = r2 >> 5;
  if (cls == 1) {
    ma &= ~((1ull << (r1 % 52)) - 1ull);
    mb &= ~((1ull << (r2 % 52)) - 1ull);
  }
  if (cls == 2) {
    ma = (r3 & 2) ? 0xfffffffffffffull : (1ull << (r1 % 52)) + ((r0 & 1) ? 1ull : 0xfffffffffffffull);
    mb = (r3 & 4) ? 0xfffffffffffffull : (1ull << (r2 % 52)) - 1ull;
  }
  if (cls == 3) {
    ea = 1500 + (int)(r1 % 40);
    eb = 1500 + (int)(r2 % 40);
  }
  *a = make_double(r0 >> 63, ea, ma);
  *b = make_double(r1 >> 63, eb, mb);
  if (cls == 4) *a = (r3 & 8) ? -0.0 : 0.0;
  if (cls == 5) {
    const int pick = (int)((r3 >> 8) % 5);
    const double sp = pick == 0 ? __longlong_as_double(0x7ff0000000000000ll)
                    : pick == 1 ? __longlong_as_double((long long)0xfff0000000000000ull)
                    : pick == 2 ? __longlong_as_double(0x7ff8000000000000ll)
                    : pick == 3 ? make_double(r0 >> 63, 0, ma)        /* subnormal */
                                : ((r3 & 16) ? -0.0 : 0.0);
    if (r3 & 32) *a = sp; else *b = sp;
  }
  if (cls == 6) *b = make_double(r1 >> 63, 1023 + (int)(r2 % 3) - 1, mb & 0xff00000000000ull);
}

__global__ void k_mul_check(unsigned long long n, unsigned long long seed, unsigned long long* bad,
                            double* first) {
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    double a, b;
    mul_operands(k, seed, &a, &b);
    const double q = shapes::mul_rn_int(a, b);
    const double ref = __dmul_rn(a, b);
    const bool same = __double_as_longlong(q) == __double_as_longlong(ref) || (q != q && ref != ref);
    if (!same && atomicAdd(bad, 1ull) == 0) {
      first[0] = a;
      first[1] = b;
    }
  }
}

/* Dependent-chain throughput of the hardware multiply and of mul_rn_int. */
template <bool INT>
__global__ void k_mul_chains(double* out, int iters) {
  double a0 = 1.0 + threadIdx.x * 1e-6, a1 = a0 + 0.25, a2 = a0 + 0.5, a3 = a0 + 0.75;
  const double c = 0.99999999999;
  for (int i = 0; i < iters; ++i) {
    if (INT) {
      a0 = shapes::mul_rn_int(a0, c); a1 = shapes::mul_rn_int(a1, c);
      a2 = shapes::mul_rn_int(a2, c); a3 = shapes::mul_rn_int(a3, c);
    } else {
      a0 = __dmul_rn(a0, c); a1 = __dmul_rn(a1, c); a2 = __dmul_rn(a2, c); a3 = __dmul_rn(a3, c);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3;
}

__global__ void k_cmp_check(const double* v, int n, unsigned long long* bad) {
  const int i = blockIdx.x, j = threadIdx.x;
  if (i >= n || j >= n) return;
  const double a = v[i], b = v[j];
  bool ok = shapes::f_le(a, b) == (a <= b) && shapes::f_lt(a, b) == (a < b);
  const double pz = shapes::plus_zero(a), ref = a + 0.0;
  ok = ok && ((__double_as_longlong(pz) == __double_as_longlong(ref)) || (pz != pz && ref != ref));
  if (!ok) atomicAdd(bad, 1ull);
}

}  // namespace

/* Compares div_rn with IEEE division on n generated operand pairs. */
extern "C" int shapes_probe_div_check(unsigned long long n, unsigned long long seed, unsigned long long* bad,
                                      double* first_ab) {
  unsigned long long* d_bad = nullptr;
  double* d_first = nullptr;
  if (cudaMalloc(&d_bad, sizeof(unsigned long long)) != cudaSuccess) return -5;
  if (cudaMalloc(&d_first, 2 * sizeof(double)) != cudaSuccess) return -5;
  cudaMemset(d_bad, 0, sizeof(unsigned long long));
  cudaMemset(d_first, 0, 2 * sizeof(double));
  k_div_check<<<152 * 16, 256>>>(n, seed, d_bad, d_first);
  cudaMemcpy(bad, d_bad, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaMemcpy(first_ab, d_first, 2 * sizeof(double), cudaMemcpyDeviceToHost);
  const cudaError_t err = cudaGetLastError();
  cudaFree(d_bad);
  cudaFree(d_first);
  return err == cudaSuccess ? 0 : -5;
}

/* Compares mul_rn_int with the hardware multiply on n generated pairs. */
extern "C" int shapes_probe_mul_check(unsigned long long n, unsigned long long seed, unsigned long long* bad,
                                      double* first_ab) {
  unsigned long long* d_bad = nullptr;
  double* d_first = nullptr;
  if (cudaMalloc(&d_bad, sizeof(unsigned long long)) != cudaSuccess) return -5;
  if (cudaMalloc(&d_first, 2 * sizeof(double)) != cudaSuccess) return -5;
  cudaMemset(d_bad, 0, sizeof(unsigned long long));
  cudaMemset(d_first, 0, 2 * sizeof(double));
  k_mul_check<<<152 * 16, 256>>>(n, seed, d_bad, d_first);
  cudaMemcpy(bad, d_bad, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaMemcpy(first_ab, d_first, 2 * sizeof(double), cudaMemcpyDeviceToHost);
  const cudaError_t err = cudaGetLastError();
  cudaFree(d_bad);
  cudaFree(d_first);
  return err == cudaSuccess ? 0 : -5;
}

/* Multiplies per second (whole GPU, 16 warps per SM, 4 chains per thread):
 * out[0] hardware, out[1] mul_rn_int. */
extern "C" int shapes_probe_mul_rate(double* out2) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -5;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -5;
  const int threads = 256, blocks = sms * 2, iters = 4000;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * threads * blocks) != cudaSuccess) return -5;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int v = 0; v < 2; ++v) {
    float ms = 0.f;
    for (int rep = 0; rep < 2; ++rep) { /* first pass warms up */
      cudaEventRecord(e0);
      if (v == 0) k_mul_chains<false><<<blocks, threads>>>(d, iters);
      else k_mul_chains<true><<<blocks, threads>>>(d, iters);
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      cudaEventElapsedTime(&ms, e0, e1);
    }
    out2[v] = ms > 0.f ? (double)blocks * threads * iters * 4.0 / (ms * 1e-3) : 0.0;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  return err == cudaSuccess ? 0 : -5;
}

/* Compares f_le/f_lt/plus_zero with IEEE on all ordered pairs of n values. */
extern "C" int shapes_probe_cmp_check(const double* host_vals, int n, unsigned long long* bad) {
  if (n <= 0 || n > 1024) return -1;
  double* d_v = nullptr;
  unsigned long long* d_bad = nullptr;
  if (cudaMalloc(&d_v, n * sizeof(double)) != cudaSuccess) return -5;
  if (cudaMalloc(&d_bad, sizeof(unsigned long long)) != cudaSuccess) return -5;
  cudaMemcpy(d_v, host_vals, n * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemset(d_bad, 0, sizeof(unsigned long long));
  k_cmp_check<<<n, n>>>(d_v, n, d_bad);
  cudaMemcpy(bad, d_bad, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  const cudaError_t err = cudaGetLastError();
  cudaFree(d_v);
  cudaFree(d_bad);
  return err == cudaSuccess ? 0 : -5;
}

/* ------------------------------------------------------------------------ */
/* tcgen05 BF16 GEMM check: D (128 x N, FP32) = A (128 x K) * B (N x K)^T    */
/* with the operand layout and descriptors of tc05.cuh, one CTA.             */
/* ------------------------------------------------------------------------ */
#include "tc05.cuh"

__global__ void k_tc05_gemm_check(const float* A, const float* B, int N, int K, float* D, int* err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tbase;
  unsigned char* sa = smem;
  unsigned char* sb = smem + 128 * 128 * 2;
  const int t = threadIdx.x;
  for (int k = 0; k < K; ++k) *reinterpret_cast<uint16_t*>(sa + tc05::kmaj(t, k, K)) = tc05::bf16_bits(A[t * K + k]);
  for (int r = t; r < N; r += 128)
    for (int k = 0; k < K; ++k) *reinterpret_cast<uint16_t*>(sb + tc05::kmaj(r, k, K)) = tc05::bf16_bits(B[r * K + k]);
  if (t == 0) tc05::mbar_init(&bar, 1);
  if (t < 32) tc05::tmem_alloc(&tbase, 256);
  tc05::fence_async_smem();
  tc05::fence_before();
  __syncthreads();
  tc05::fence_after();
  const uint32_t base = tbase;
  if (t == 0) {
    tc05::gemm(base, tc05::smem_addr(sa), tc05::smem_addr(sb), 128, N, K, false);
    tc05::commit(&bar);
  }
  const bool ok = tc05::mbar_wait(&bar, 0);
  if (!ok && (t & 31) == 0) atomicExch(err, 1);
  tc05::fence_after();
  const int w = t >> 5;
  for (int c = 0; c < N; c += 16) {
    float v[16];
    tc05::tmem_ld16(tc05::taddr(base, 32 * w, c), v);
    for (int k = 0; k < 16; ++k) D[t * N + c + k] = ok ? v[k] : 0.f;
  }
  tc05::fence_before();
  __syncthreads();
  if (t < 32) tc05::tmem_free(base, 256);
}

extern "C" int shapes_probe_tc05_gemm(const float* A, const float* B, int N, int K, float* D) {
  if (N < 16 || N > 256 || (N & 15) || K < 16 || K > 128 || (K & 15)) return -1;
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  int* dErr = nullptr;
  cudaError_t e = cudaMalloc(&dA, sizeof(float) * 128 * K);
  if (e == cudaSuccess) e = cudaMalloc(&dB, sizeof(float) * N * K);
  if (e == cudaSuccess) e = cudaMalloc(&dD, sizeof(float) * 128 * N);
  if (e == cudaSuccess) e = cudaMalloc(&dErr, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(dErr, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(dA, A, sizeof(float) * 128 * K, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dB, B, sizeof(float) * N * K, cudaMemcpyHostToDevice);
  const int smem = 128 * 128 * 2 + 256 * 128 * 2 + 16384; /* operands + slack */
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tc05_gemm_check, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) {
    k_tc05_gemm_check<<<1, 128, smem>>>(dA, dB, N, K, dD, dErr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&herr, dErr, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(D, dD, sizeof(float) * 128 * N, cudaMemcpyDeviceToHost);
  cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(dErr);
  if (e != cudaSuccess) return -5;
  return herr ? -6 : 0;
}

/* ---- add_rn_int: checks against the hardware addition and throughput ---- */

__host__ __device__ __forceinline__ double bits_to_double(unsigned long long u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double d;
  __builtin_memcpy(&d, &u, 8);
  return d;
#endif
}

__host__ __device__ __forceinline__ unsigned long long double_to_bits(double d) {
#if defined(__CUDA_ARCH__)
  return (unsigned long long)__double_as_longlong(d);
#else
  unsigned long long u;
  __builtin_memcpy(&u, &d, 8);
  return u;
#endif
}

/* Operand classes for add_rn_int: random exponents over the fast range and
 * beyond it, close exponents, near and exact cancellation, shifts past the
 * significand, neighbours of the rounding midpoint, powers of two, all-ones
 * significands, and zeros, subnormals, infinities and NaN. */
__host__ __device__ void add_operands(unsigned long long k, unsigned long long seed, double* a, double* b) {
  const unsigned long long r0 = mix64(k ^ seed), r1 = mix64(r0), r2 = mix64(r1), r3 = mix64(r2);
  const int cls = (int)(r3 % 10);
  long long ea = 40 + (long long)(r1 % 1970), eb;
  unsigned long long ma = r0, mb = r2 >> 3;
  switch (cls) {
    case 0: eb = 40 + (long long)(r2 % 1970); break;
    case 1: eb = ea + (long long)(r2 % 7) - 3; break;
    case 2: eb = ea; mb = ma ^ (r2 & 0xffull); break;
    case 3: eb = ea - (long long)(r2 % 70); break;
    case 4: eb = ea - 53 - (long long)(r2 % 3); ma &= ~0xfffull; break;
    case 5: eb = ea - (long long)(r2 % 60); mb = 1ull << (r2 % 52); break;
    case 6: eb = ea; mb = ma; break;
    case 7: eb = ea - 1 - (long long)(r2 % 5); ma = 0xfffffffffffffull; mb = 0xfffffffffffffull; break;
    default: eb = 40 + (long long)(r2 % 1970); break;
  }
  if (eb < 1) eb = 1;
  if (eb > 2046) eb = 2046;
  *a = bits_to_double(((r0 >> 63) << 63) | ((unsigned long long)ea << 52) | (ma & 0xfffffffffffffull));
  *b = bits_to_double(((r1 >> 63) << 63) | ((unsigned long long)eb << 52) | (mb & 0xfffffffffffffull));
  if (cls >= 8) {
    const int pick = (int)((r3 >> 8) % 6);
    const unsigned long long sp = pick == 0 ? 0x7ff0000000000000ull
                                : pick == 1 ? 0xfff0000000000000ull
                                : pick == 2 ? 0x7ff8000000000000ull
                                : pick == 3 ? ((r0 >> 63) << 63) | (ma & 0xfffffffffffffull) /* subnormal */
                                : pick == 4 ? ((r3 & 16) ? 0x8000000000000000ull : 0ull)
                                            : 0x7fefffffffffffffull;
    if (r3 & 32) *a = bits_to_double(sp); else *b = bits_to_double(sp);
  }
  if (r3 & 0x100) {
    const double t = *a;
    *a = *b;
    *b = t;
  }
}

__global__ void k_add_check(unsigned long long n, unsigned long long seed, unsigned long long* bad,
                            double* first) {
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    double a, b;
    add_operands(k, seed, &a, &b);
    const double q = shapes::add_rn_int(a, b);
    const double ref = __dadd_rn(a, b);
    const bool same = __double_as_longlong(q) == __double_as_longlong(ref) || (q != q && ref != ref);
    if (!same && atomicAdd(bad, 1ull) == 0) {
      first[0] = a;
      first[1] = b;
    }
  }
}

extern "C" int shapes_probe_add_check(unsigned long long n, unsigned long long seed, unsigned long long* bad,
                                      double* first_ab) {
  unsigned long long* d_bad = nullptr;
  double* d_first = nullptr;
  if (cudaMalloc(&d_bad, sizeof(unsigned long long)) != cudaSuccess) return -5;
  if (cudaMalloc(&d_first, 2 * sizeof(double)) != cudaSuccess) return -5;
  cudaMemset(d_bad, 0, sizeof(unsigned long long));
  cudaMemset(d_first, 0, 2 * sizeof(double));
  k_add_check<<<152 * 16, 256>>>(n, seed, d_bad, d_first);
  cudaMemcpy(bad, d_bad, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaMemcpy(first_ab, d_first, 2 * sizeof(double), cudaMemcpyDeviceToHost);
  const cudaError_t err = cudaGetLastError();
  cudaFree(d_bad);
  cudaFree(d_first);
  return err == cudaSuccess ? 0 : -5;
}

/* The same integer steps on the host against the host's own addition (no
 * GPU needed): n pairs from the same operand classes. */
extern "C" int shapes_probe_add_check_host(unsigned long long n, unsigned long long seed, unsigned long long* bad,
                                           double* first_ab) {
  unsigned long long nb = 0;
  for (unsigned long long k = 0; k < n; ++k) {
    double a, b;
    add_operands(k, seed, &a, &b);
    const double q = shapes::add_rn_int(a, b);
    volatile double va = a, vb = b;
    const double ref = va + vb;
    const bool same = double_to_bits(q) == double_to_bits(ref) || (q != q && ref != ref);
    if (!same && nb++ == 0) {
      first_ab[0] = a;
      first_ab[1] = b;
    }
  }
  *bad = nb;
  return 0;
}

/* Sums per second (whole GPU) of independent chains: NF on the FP64 pipe and
 * NI through add_rn_int in the same warps, and the same split for products
 * (mul_rn_int).  out6: adds {FP64 only, integer only, 4 + 4 mixed}, products
 * {FP64 only, integer only, 4 + 4 mixed}. */
template <int NF, int NI, bool ADD>
__global__ void k_split_chains(double* out, int iters) {
  double f[NF > 0 ? NF : 1], g[NI > 0 ? NI : 1];
#pragma unroll
  for (int k = 0; k < NF; ++k) f[k] = 1.0 + threadIdx.x * 1e-6 + 0.1 * k;
#pragma unroll
  for (int k = 0; k < NI; ++k) g[k] = 1.25 + threadIdx.x * 1e-6 + 0.1 * k;
  const double c = ADD ? 1.0000000001 : 0.99999999999;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < NF; ++k) f[k] = ADD ? __dadd_rn(f[k], c) : __dmul_rn(f[k], c);
#pragma unroll
    for (int k = 0; k < NI; ++k) g[k] = ADD ? shapes::add_rn_int(g[k], c) : shapes::mul_rn_int(g[k], c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < NF; ++k) s += f[k];
#pragma unroll
  for (int k = 0; k < NI; ++k) s += g[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <int NF, int NI, bool ADD>
static double split_rate(double* d, int blocks, int threads) {
  const int iters = 2000;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float ms = 0.f;
  for (int rep = 0; rep < 2; ++rep) {
    cudaEventRecord(e0);
    k_split_chains<NF, NI, ADD><<<blocks, threads>>>(d, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms > 0.f ? (double)blocks * threads * iters * (NF + NI) / (ms * 1e-3) : 0.0;
}

extern "C" int shapes_probe_split_rates(double* out6) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -5;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -5;
  const int threads = 256, blocks = sms * 4;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * threads * blocks) != cudaSuccess) return -5;
  out6[0] = split_rate<8, 0, true>(d, blocks, threads);
  out6[1] = split_rate<0, 8, true>(d, blocks, threads);
  out6[2] = split_rate<4, 4, true>(d, blocks, threads);
  out6[3] = split_rate<8, 0, false>(d, blocks, threads);
  out6[4] = split_rate<0, 8, false>(d, blocks, threads);
  out6[5] = split_rate<4, 4, false>(d, blocks, threads);
  const cudaError_t err = cudaGetLastError();
  cudaFree(d);
  return err == cudaSuccess ? 0 : -5;
}

/* ---- ticket order of the ordered large-world solve (lw_order.cuh), on the host ---- */
#include <algorithm>
#include <vector>

#include "lw_order.cuh"

/* For every P <= max_p, R <= max_r and skew 1 <= S <= R: lw_ticket(t) for each
 * ticket t against the tickets sorted by key p S + r (ties by p).  *cases is
 * the number of tickets checked, *bad the number that differ. */
extern "C" int shapes_probe_lw_ticket_check(int max_p, int max_r, unsigned long long* cases, unsigned long long* bad) {
  unsigned long long n = 0, nbad = 0;
  std::vector<std::pair<long long, int>> order;
  for (int P = 1; P <= max_p; ++P)
    for (int R = 1; R <= max_r; ++R)
      for (int S = 1; S <= R; ++S) {
        order.clear();
        for (int p = 0; p < P; ++p)
          for (int r = 0; r < R; ++r) order.push_back({(long long)p * S + r, p * R + r});
        std::stable_sort(order.begin(), order.end(),
                         [](const std::pair<long long, int>& x, const std::pair<long long, int>& y) {
                           return x.first < y.first;
                         });
        for (long long t = 0; t < (long long)P * R; ++t) {
          int p, r;
          shapes::lw_ticket(t, P, S, R, p, r);
          ++n;
          if (p * R + r != order[(size_t)t].second) ++nbad;
        }
      }
  *cases = n;
  *bad = nbad;
  return 0;
}
