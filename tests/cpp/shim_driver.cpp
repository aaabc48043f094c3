// Drives the reference-spelled launchers of skinny.hpp the way the reference's test harness calls
// its variants (test.cu:114-143): device buffers, one call per variant, results copied back.
// Prints "name sum_of_C" lines; the Python test compares them with the oracle on the same data.
#include <cuda_runtime.h>

#include <cstdio>
#include <vector>

#include "skinny.hpp"

template <typename F>
static void run(const char* name, F f, int K, int M, int N, bool tsmm) {
  std::vector<double> hA((size_t)K * M), hB(tsmm ? (size_t)M * N : (size_t)K * N), hC(tsmm ? (size_t)K * N : M * N);
  for (size_t i = 0; i < hA.size(); i++) hA[i] = (double)((i * 7 + 3) % 11) - 5.0;
  for (size_t i = 0; i < hB.size(); i++) hB[i] = (double)((i * 5 + 1) % 9) - 4.0;
  for (size_t i = 0; i < hC.size(); i++) hC[i] = (double)(i % 5) - 2.0;
  double *A, *B, *C;
  cudaMalloc(&A, hA.size() * 8);
  cudaMalloc(&B, hB.size() * 8);
  cudaMalloc(&C, hC.size() * 8);
  cudaMemcpy(A, hA.data(), hA.size() * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(B, hB.data(), hB.size() * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(C, hC.data(), hC.size() * 8, cudaMemcpyHostToDevice);
  const bool ok = f(A, B, C);
  cudaDeviceSynchronize();
  cudaMemcpy(hC.data(), C, hC.size() * 8, cudaMemcpyDeviceToHost);
  double s = 0;
  for (double x : hC) s += x;
  std::printf("%s %d %.17g\n", name, ok ? 1 : 0, s);
  cudaFree(A);
  cudaFree(B);
  cudaFree(C);
}

int main() {
  const int K = 10000;
  run("GENV5_8x8", [&](double* A, double* B, double* C) {
    return GENV5::tsmttsm<double, 8, 8>(52, 8, 8, K, A, 8, 1.0, B, 8, 0.5, C, 8);
  }, K, 8, 8, false);
  run("SPECSMALL_PQ_4x4", [&](double* A, double* B, double* C) {
    return SPECSMALL::tsmttsm<double, skinny::PseudoQuad, 4, 4>(52, 4, 4, K, A, 4, 1.0, B, 4, 0.5, C, 4);
  }, K, 4, 4, false);
  run("GENV3_GLOBAL_2x3", [&](double* A, double* B, double* C) {
    return GENV3::tsmttsm<double, double, 2, 3, GENV3::MEMPATH::GLOBAL>(52, 2, 3, K, A, 2, 1.0, B, 3, 0.5, C, 2);
  }, K, 2, 3, false);
  run("MISMATCH", [&](double* A, double* B, double* C) {
    return GENV5::tsmttsm<double, 8, 8>(52, 4, 4, K, A, 4, 1.0, B, 4, 0.5, C, 4);
  }, K, 4, 4, false);
  run("FIX3_4x4", [&](double* A, double* B, double* C) {
    return tsmm_fix3<double, 4, 4>(52, 4, 4, K, A, 4, 1.0, B, 4, 0.5, C, 4);
  }, K, 4, 4, true);
  run("VAR1_3x5", [&](double* A, double* B, double* C) {
    return tsmm_var1<double>(52, 3, 5, K, A, 3, 1.0, B, 3, 0.5, C, 5);
  }, K, 3, 5, true);
  return 0;
}
