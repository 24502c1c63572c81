// div_check_gpu.cu -- the device build of huji-rich_gb300/csrc/rg_div.cuh
// against the device's IEEE division (a / b), bit for bit.
//
//   div_check_gpu <cases per family> <rng seed>
//
// 1. Every operand pair of tests/div_cases.h (generated on the host) is
//    divided on the device by rg::div_rn and by a / b; the results are
//    compared bitwise on the host (NaN against NaN).
// 2. The FP32 reciprocal approximation the fast path starts from is checked
//    on every float f in [1, 2): max |1 - f * rcp(f)| (the fast path needs
//    at most 2^-22 and falls back above it).
// 3. Throughput: 64 divisions per thread over 152 * 8 blocks of 256 threads,
//    rg::div_rn against a / b, timed with CUDA events.
// 4. The same for the square root: rg::sqrt_rn against sqrt on the families
//    of divcases::generate_sqrt, the FP32 reciprocal square root
//    approximation on every float in [1, 4), and the throughput.
// Prints one JSON line.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "div_cases.h"
#include "rg_div.cuh"

#define CK(x)                                                                  \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess) {                                                   \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));            \
      std::exit(3);                                                            \
    }                                                                          \
  } while (0)

__global__ void k_divide(const double* a, const double* b, double* q_new, double* q_ref, unsigned char* fast,
                         long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double q;
    const bool f = rg::div_rn_fast(a[i], b[i], rg::RcpSeedDevice{}, &q);
    q_new[i] = f ? q : a[i] / b[i];
    fast[i] = f ? 1 : 0;
    q_ref[i] = a[i] / b[i];
  }
}

// max over f in [1, 2) of |1 - f * rcp(f)|, as the bits of a non-negative double
__global__ void k_rcp_error(unsigned long long* worst) {
  const unsigned m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= (1u << 23)) return;
  const float f = __uint_as_float(0x3f800000u | m);
  const float r = rg::RcpSeedDevice{}(f);
  const double e = fabs(1.0 - static_cast<double>(f) * static_cast<double>(r));
  atomicMax(worst, static_cast<unsigned long long>(__double_as_longlong(e)));
}

__global__ void k_sqrt(const double* x, double* r_new, double* r_ref, unsigned char* fast, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double r;
    const bool f = rg::sqrt_rn_fast(x[i], rg::RsqrtSeedDevice{}, &r);
    r_new[i] = f ? r : sqrt(x[i]);
    fast[i] = f ? 1 : 0;
    r_ref[i] = sqrt(x[i]);
  }
}

// max over f in [1, 4) of |1 - f * rsqrt(f)^2|
__global__ void k_rsqrt_error(unsigned long long* worst) {
  const unsigned m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= (1u << 24)) return;
  const float f = __uint_as_float((0x3f800000u + (m >> 23 << 23)) | (m & 0x7fffffu));
  const float y = rg::RsqrtSeedDevice{}(f);
  const double e = fabs(1.0 - static_cast<double>(f) * static_cast<double>(y) * static_cast<double>(y));
  atomicMax(worst, static_cast<unsigned long long>(__double_as_longlong(e)));
}

template <bool kNew>
__global__ void k_sqrt_throughput(const double* a, unsigned long long* sink) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned long long ua = static_cast<unsigned long long>(__double_as_longlong(fabs(a[t])));
  unsigned long long acc = 0;
#pragma unroll 4
  for (int k = 0; k < 64; ++k) {
    const double x = __longlong_as_double(static_cast<long long>(ua + 977ull * k));
    const double r = kNew ? rg::sqrt_rn(x) : sqrt(x);
    acc ^= static_cast<unsigned long long>(__double_as_longlong(r));
  }
  sink[t] = acc;
}

template <bool kNew>
__global__ void k_throughput(const double* a, const double* b, unsigned long long* sink) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned long long ua = static_cast<unsigned long long>(__double_as_longlong(a[t]));
  const unsigned long long ub = static_cast<unsigned long long>(__double_as_longlong(b[t]));
  unsigned long long acc = 0;
#pragma unroll 4
  for (int k = 0; k < 64; ++k) {
    // both operands change every iteration (nothing to hoist out of the loop)
    const double x = __longlong_as_double(static_cast<long long>(ua + 977ull * k));
    const double y = __longlong_as_double(static_cast<long long>(ub + 1237ull * k));
    const double q = kNew ? rg::div_rn(x, y) : x / y;
    acc ^= static_cast<unsigned long long>(__double_as_longlong(q));
  }
  sink[t] = acc;
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: div_check_gpu <cases per family> <rng seed>\n");
    return 2;
  }
  const long long per = std::atoll(argv[1]);
  std::mt19937_64 rng(std::strtoull(argv[2], nullptr, 10));
  std::vector<double> ha, hb;
  divcases::generate(rng, per, [&](double a, double b) {
    ha.push_back(a);
    hb.push_back(b);
  });
  const long long n = static_cast<long long>(ha.size());
  double *a, *b, *qn, *qr;
  unsigned char* fast;
  CK(cudaMalloc(&a, n * sizeof(double)));
  CK(cudaMalloc(&b, n * sizeof(double)));
  CK(cudaMalloc(&qn, n * sizeof(double)));
  CK(cudaMalloc(&qr, n * sizeof(double)));
  CK(cudaMalloc(&fast, n));
  CK(cudaMemcpy(a, ha.data(), n * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b, hb.data(), n * sizeof(double), cudaMemcpyHostToDevice));
  k_divide<<<152 * 16, 256>>>(a, b, qn, qr, fast, n);
  CK(cudaGetLastError());
  std::vector<double> hn(n), hr(n);
  std::vector<unsigned char> hf(n);
  CK(cudaMemcpy(hn.data(), qn, n * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hr.data(), qr, n * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hf.data(), fast, n, cudaMemcpyDeviceToHost));
  long long bad = 0, nfast = 0;
  double bad_a = 0, bad_b = 0;
  for (long long i = 0; i < n; ++i) {
    nfast += hf[i];
    const bool nan_n = hn[i] != hn[i], nan_r = hr[i] != hr[i];
    if (!(divcases::bits(hn[i]) == divcases::bits(hr[i]) || (nan_n && nan_r))) {
      if (!bad) {
        bad_a = ha[i];
        bad_b = hb[i];
      }
      ++bad;
    }
  }
  // the seed's error on [1, 2)
  unsigned long long* worst;
  CK(cudaMalloc(&worst, sizeof *worst));
  CK(cudaMemset(worst, 0, sizeof *worst));
  k_rcp_error<<<(1 << 23) / 256, 256>>>(worst);
  unsigned long long hw = 0;
  CK(cudaMemcpy(&hw, worst, sizeof hw, cudaMemcpyDeviceToHost));
  double rcp_err;
  std::memcpy(&rcp_err, &hw, sizeof rcp_err);
  // throughput (operands: the moderate-size family, which starts at 2 * per)
  const int blocks = 152 * 8, threads = 256, lanes = blocks * threads;
  unsigned long long* sink;
  CK(cudaMalloc(&sink, lanes * sizeof(unsigned long long)));
  const long long off = 2 * per + lanes <= n ? 2 * per : 0;
  cudaEvent_t e0, e1, e2;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventCreate(&e2));
  k_throughput<true><<<blocks, threads>>>(a + off, b + off, sink);
  k_throughput<false><<<blocks, threads>>>(a + off, b + off, sink);
  CK(cudaEventRecord(e0));
  k_throughput<true><<<blocks, threads>>>(a + off, b + off, sink);
  CK(cudaEventRecord(e1));
  k_throughput<false><<<blocks, threads>>>(a + off, b + off, sink);
  CK(cudaEventRecord(e2));
  CK(cudaEventSynchronize(e2));
  float ms_new = 0, ms_ref = 0;
  CK(cudaEventElapsedTime(&ms_new, e0, e1));
  CK(cudaEventElapsedTime(&ms_ref, e1, e2));
  const double divs = 64.0 * lanes;
  // square roots
  std::vector<double> hx;
  divcases::generate_sqrt(rng, per, [&](double x) { hx.push_back(x); });
  const long long ns = static_cast<long long>(hx.size());
  double *x, *rn, *rr;
  unsigned char* sfast;
  CK(cudaMalloc(&x, ns * sizeof(double)));
  CK(cudaMalloc(&rn, ns * sizeof(double)));
  CK(cudaMalloc(&rr, ns * sizeof(double)));
  CK(cudaMalloc(&sfast, ns));
  CK(cudaMemcpy(x, hx.data(), ns * sizeof(double), cudaMemcpyHostToDevice));
  k_sqrt<<<152 * 16, 256>>>(x, rn, rr, sfast, ns);
  CK(cudaGetLastError());
  std::vector<double> hsn(ns), hsr(ns);
  std::vector<unsigned char> hsf(ns);
  CK(cudaMemcpy(hsn.data(), rn, ns * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hsr.data(), rr, ns * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hsf.data(), sfast, ns, cudaMemcpyDeviceToHost));
  long long sbad = 0, sfastn = 0;
  double sbad_x = 0;
  for (long long i = 0; i < ns; ++i) {
    sfastn += hsf[i];
    const bool nan_n = hsn[i] != hsn[i], nan_r = hsr[i] != hsr[i];
    if (!(divcases::bits(hsn[i]) == divcases::bits(hsr[i]) || (nan_n && nan_r))) {
      if (!sbad) sbad_x = hx[i];
      ++sbad;
    }
  }
  CK(cudaMemset(worst, 0, sizeof *worst));
  k_rsqrt_error<<<(1 << 24) / 256, 256>>>(worst);
  CK(cudaMemcpy(&hw, worst, sizeof hw, cudaMemcpyDeviceToHost));
  double rsqrt_err;
  std::memcpy(&rsqrt_err, &hw, sizeof rsqrt_err);
  k_sqrt_throughput<true><<<blocks, threads>>>(a + off, sink);
  k_sqrt_throughput<false><<<blocks, threads>>>(a + off, sink);
  CK(cudaEventRecord(e0));
  k_sqrt_throughput<true><<<blocks, threads>>>(a + off, sink);
  CK(cudaEventRecord(e1));
  k_sqrt_throughput<false><<<blocks, threads>>>(a + off, sink);
  CK(cudaEventRecord(e2));
  CK(cudaEventSynchronize(e2));
  float sms_new = 0, sms_ref = 0;
  CK(cudaEventElapsedTime(&sms_new, e0, e1));
  CK(cudaEventElapsedTime(&sms_ref, e1, e2));
  std::printf("{\"cases\": %lld, \"mismatches\": %lld, \"fast\": %lld, \"first_a\": %.17g, \"first_b\": %.17g, "
              "\"rcp_max_rel_error\": %.6g, \"div_rn_gdiv_per_s\": %.4g, \"ieee_div_gdiv_per_s\": %.4g, "
              "\"sqrt_cases\": %lld, \"sqrt_mismatches\": %lld, \"sqrt_fast\": %lld, \"sqrt_first_x\": %.17g, "
              "\"rsqrt_max_rel_error\": %.6g, \"sqrt_rn_gsqrt_per_s\": %.4g, \"ieee_sqrt_gsqrt_per_s\": %.4g}\n",
              n, bad, nfast, bad_a, bad_b, rcp_err, divs / (ms_new * 1e6), divs / (ms_ref * 1e6), ns, sbad, sfastn,
              sbad_x, rsqrt_err, divs / (sms_new * 1e6), divs / (sms_ref * 1e6));
  return bad == 0 && sbad == 0 ? 0 : 1;
}
