"""The C ABI used from a C program on the GPU, with no Python or torch in the
process: it allocates device buffers with the CUDA runtime, sizes and passes
a workspace, runs fsk_kde16 (tensor-core path and the fp32_ieee path) and
fsk_kde16_noalloc on a stream of its own, reads fsk_device_status and checks
the densities against a double-precision sum on the host (relative 1e-5)."""
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent

C_SRC = r"""
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <cuda_runtime.h>
#include "fsk.h"

#define N 3001
#define M 257
#define D 16

static double ref_density(const float* x, const float* q, double h) {
  const double norm = 1.0 / (pow(2.0 * M_PI, D / 2.0) * pow(h, D) * N);
  double s = 0.0;
  for (int j = 0; j < N; ++j) {
    double d2 = 0.0;
    for (int k = 0; k < D; ++k) {
      const double t = (double)q[k] - (double)x[j * D + k];
      d2 += t * t;
    }
    s += exp(-d2 / (2.0 * h * h));
  }
  return s * norm;
}

int main(void) {
  float* x = (float*)malloc(sizeof(float) * N * D);
  float* q = (float*)malloc(sizeof(float) * M * D);
  float* out = (float*)malloc(sizeof(float) * M);
  unsigned int seed = 12345u;
  for (int i = 0; i < N * D; ++i) { seed = seed * 1664525u + 1013904223u; x[i] = (float)((seed >> 8) * (1.0 / 16777216.0)) * 4.0f - 2.0f; }
  for (int i = 0; i < M * D; ++i) { seed = seed * 1664525u + 1013904223u; q[i] = (float)((seed >> 8) * (1.0 / 16777216.0)) * 4.0f - 2.0f; }
  const double h = 0.9;
  const double scale = 1.0 / (pow(2.0 * M_PI, D / 2.0) * pow(h, D) * N);
  float *dx, *dq, *dout;
  void* ws;
  cudaStream_t s;
  if (cudaStreamCreate(&s) != cudaSuccess) return 10;
  cudaMalloc((void**)&dx, sizeof(float) * N * D);
  cudaMalloc((void**)&dq, sizeof(float) * M * D);
  cudaMalloc((void**)&dout, sizeof(float) * M);
  cudaMemcpy(dx, x, sizeof(float) * N * D, cudaMemcpyHostToDevice);
  cudaMemcpy(dq, q, sizeof(float) * M * D, cudaMemcpyHostToDevice);
  const int flags[2] = {0, FSK_PREC_IEEE};
  double worst = 0.0;
  for (int f = 0; f < 3; ++f) {
    int st;
    if (f < 2) {
      const size_t bytes = fsk_kde16_workspace_bytes(M, N, flags[f]);
      if (cudaMalloc(&ws, bytes) != cudaSuccess) return 11;
      st = fsk_kde16(dq, M, dx, N, h, flags[f], scale, 0.0, dout, ws, bytes, (void*)s);
      if (st == FSK_OK) st = fsk_device_status((void*)s);
      cudaFree(ws);
    } else {
      st = fsk_kde16_noalloc(dq, M, dx, N, h, 0, scale, 0.0, dout, (void*)s);
      if (st == FSK_OK) st = fsk_device_status((void*)s);
    }
    if (st != FSK_OK) { printf("status %d: %s\n", st, fsk_strerror(st)); return 12 + f; }
    cudaMemcpy(out, dout, sizeof(float) * M, cudaMemcpyDeviceToHost);
    for (int i = 0; i < M; i += 16) {
      const double r = ref_density(x, q + i * D, h);
      const double e = fabs((double)out[i] - r) / r;
      if (e > worst) worst = e;
    }
  }
  printf("max rel err %.3e\n", worst);
  return worst < 1e-5 ? 0 : 20;
}
"""


def test_c_program_runs_the_kde_on_the_gpu(cuda_dev, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    from fsk import _build

    lib = _build.build()
    src = tmp_path / "consumer.c"
    src.write_text(C_SRC)
    exe = tmp_path / "consumer"
    subprocess.run([nvcc, "-x", "c", str(src), "-I", str(ROOT / "include"), "-o", str(exe),
                    "-L", str(lib.parent), "-lfsk", "-lm", f"-Xlinker=-rpath,{lib.parent}"], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, (res.returncode, res.stdout, res.stderr)
    assert "max rel err" in res.stdout
