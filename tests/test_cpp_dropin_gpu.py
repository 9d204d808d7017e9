"""The C++ drop-in header end to end on the GPU: a program written against the
reference's host API (kronmult6_batched, kronmult4_xbatched, kgemm_nn_batched
with the reference's argument lists) is compiled with g++, linked against the
library, run, and its results are checked against the reference's golden
vectors and the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests.common import blockwise_rel_err, golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")

PROGRAM = r'''
#include <cuda_runtime.h>
#include <cstdio>
#include <vector>
#include "kronmult_gb300.hpp"

// ramp inputs of test_kronmult6_batched.cpp:148-175 (as the golden vectors use them)
static void ramp(int n, int d, int batch, std::vector<double>& A, std::vector<double>& X) {
  int N = 1;
  for (int l = 0; l < d; ++l) N *= n;
  A.assign((size_t)n * n * d * batch, 0.0);
  X.assign((size_t)N * batch, 0.0);
  const double sa = (double)n * n * d * batch, sx = (double)N * batch;
  for (int kb = 0; kb < batch; ++kb)
    for (int l = 0; l < d; ++l)
      for (int j = 1; j <= n; ++j)
        for (int i = 1; i <= n; ++i)
          A[((size_t)kb * d + l) * n * n + (i - 1) + (size_t)(j - 1) * n] =
              (i + (j - 1) * n + l * n * n + kb * batch) / sa;
  for (int k = 1; k <= batch; ++k)
    for (int i = 1; i <= N; ++i) X[(size_t)(k - 1) * N + (i - 1)] = (i + (k - 1) * (double)N) / sx;
}

int main(int argc, char** argv) {
  const int n = 4, d = 6, batch = 3, N = 4096;
  std::vector<double> A, X;
  ramp(n, d, batch, A, X);
  double *dA, *dX, *dY, *dW;
  cudaMalloc(&dA, A.size() * 8);
  cudaMalloc(&dX, X.size() * 8);
  cudaMalloc(&dY, X.size() * 8);
  cudaMalloc(&dW, X.size() * 8);
  cudaMemcpy(dA, A.data(), A.size() * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(dX, X.data(), X.size() * 8, cudaMemcpyHostToDevice);
  cudaMemset(dY, 0, X.size() * 8);
  kronmult6_batched(n, dA, dX, dY, dW, batch);   // the reference's call, unchanged
  cudaDeviceSynchronize();
  std::vector<double> Y(X.size());
  cudaMemcpy(Y.data(), dY, Y.size() * 8, cudaMemcpyDeviceToHost);
  FILE* f = fopen(argv[1], "wb");
  fwrite(Y.data(), 8, Y.size(), f);
  // kgemm_nn_batched with the reference test's alpha/beta: C = 1.3*A*B + 1.2*C
  const int mm = 8, nn = 15, kk = 22, nb = 2;
  std::vector<double> Ag((size_t)mm * kk * nb), Bg((size_t)kk * nn * nb), Cg((size_t)mm * nn * nb, 1.0);
  for (size_t i = 0; i < Ag.size(); ++i) Ag[i] = 0.25 * (double)(i % 7) - 0.5;
  for (size_t i = 0; i < Bg.size(); ++i) Bg[i] = 0.125 * (double)(i % 5) + 0.1;
  double *gA, *gB, *gC;
  cudaMalloc(&gA, Ag.size() * 8);
  cudaMalloc(&gB, Bg.size() * 8);
  cudaMalloc(&gC, Cg.size() * 8);
  cudaMemcpy(gA, Ag.data(), Ag.size() * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(gB, Bg.data(), Bg.size() * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(gC, Cg.data(), Cg.size() * 8, cudaMemcpyHostToDevice);
  double* hp[3][2] = {{gA, gA + mm * kk}, {gB, gB + kk * nn}, {gC, gC + mm * nn}};
  int hld[3][2] = {{mm, mm}, {kk, kk}, {mm, mm}};
  double** dp[3];
  int* dld[3];
  for (int q = 0; q < 3; ++q) {
    cudaMalloc(&dp[q], sizeof(hp[q]));
    cudaMemcpy(dp[q], hp[q], sizeof(hp[q]), cudaMemcpyHostToDevice);
    cudaMalloc(&dld[q], sizeof(hld[q]));
    cudaMemcpy(dld[q], hld[q], sizeof(hld[q]), cudaMemcpyHostToDevice);
  }
  kgemm_nn_batched(mm, nn, kk, 1.3, dp[0], dld[0], dp[1], dld[1], 1.2, dp[2], dld[2], nb);
  cudaDeviceSynchronize();
  cudaMemcpy(Cg.data(), gC, Cg.size() * 8, cudaMemcpyDeviceToHost);
  fwrite(Ag.data(), 8, Ag.size(), f);
  fwrite(Bg.data(), 8, Bg.size(), f);
  fwrite(Cg.data(), 8, Cg.size(), f);
  fclose(f);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
'''


@pytest.fixture(scope="module")
def program(kmx, tmp_path_factory):
    if shutil.which("g++") is None or not os.path.isdir(os.path.join(CUDA, "include")):
        pytest.skip("g++ or the CUDA toolkit headers are missing")
    d = tmp_path_factory.mktemp("dropin")
    src = d / "user.cpp"
    src.write_text(PROGRAM)
    exe = d / "user"
    lib_dir = os.path.join(ROOT, "kronmult_gb300")
    subprocess.run(["g++", "-std=c++14", "-O2", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(CUDA, "include"), str(src), "-o", str(exe),
                    f"-L{lib_dir}", "-lkronmult_gb300", f"-Wl,-rpath,{lib_dir}",
                    f"-L{os.path.join(CUDA, 'lib64')}", "-lcudart",
                    f"-Wl,-rpath,{os.path.join(CUDA, 'lib64')}"], check=True)
    return exe, d


def test_cpp_program_matches_golden_and_oracle(program, oracle):
    exe, d = program
    out = d / "out.bin"
    subprocess.run([str(exe), str(out)], check=True, timeout=120)
    raw = np.fromfile(out, dtype=np.float64)
    N, batch = 4096, 3
    Y = raw[: N * batch].reshape(batch, N)
    assert blockwise_rel_err(Y, golden()["batched_d6_n4_b3"]) <= 1e-13
    mm, nn, kk, nb = 8, 15, 22, 2
    o = N * batch
    Ag = raw[o: o + mm * kk * nb]
    o += mm * kk * nb
    Bg = raw[o: o + kk * nn * nb]
    o += kk * nn * nb
    Cg = raw[o: o + mm * nn * nb]
    ref = np.ones(mm * nn * nb)
    oracle.kgemm_batched("nn", mm, nn, kk, 1.3, Ag, [0, mm * kk], [mm, mm], Bg, [0, kk * nn],
                         [kk, kk], 1.2, ref, [0, mm * nn], [mm, mm])
    assert blockwise_rel_err(Cg.reshape(nb, -1), ref.reshape(nb, -1)) <= 1e-13
