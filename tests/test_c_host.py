"""The C ABI from a C host (no Python in the call path): a C11 program that
includes include/scarf_gb300.h compiles cleanly, links against
libscarfgpu.so, and on a machine without a GPU gets a status and an error
message back from sg_create instead of a crash (no CPU fallback)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include "scarf_gb300.h"

int main(void) {
  sg_handle* h = NULL;
  int rc = sg_create(0, 0, &h);
  printf("version %d\n", sg_version());
  if (rc != 0) {
    const char* msg = sg_last_error();
    printf("create %d: %s\n", rc, msg ? msg : "(none)");
    return 0;
  }
  sg_destroy(h);
  printf("create ok\n");
  return 0;
}
"""


def test_c_program_builds_links_and_reports(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    from scarf_gb300 import build
    try:
        lib = build.build()
    except RuntimeError as e:  # pragma: no cover - nvcc absent
        pytest.skip(f"cannot build: {e}")
    src = tmp_path / "host.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "host"
    r = subprocess.run([gcc, "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror", str(src), "-I",
                        os.path.join(ROOT, "include"), "-L", str(lib.parent), "-lscarfgpu",
                        f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.startswith("version ")
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        assert "create -" in out.stdout and "(none)" not in out.stdout


KNN_PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include <cuda_runtime.h>
#include "scarf_gb300.h"

#define N 600
#define D 12
#define LD 12
#define K 7

int main(void) {
  static float pts[N * LD];
  unsigned s = 12345u;
  for (int i = 0; i < N * LD; ++i) {   /* a fixed LCG, clustered by row parity */
    s = s * 1664525u + 1013904223u;
    pts[i] = (float)(s >> 8) / 16777216.0f + (float)((i / LD) % 2) * 3.0f;
  }
  sg_handle* h = NULL;
  if (sg_create(0, 0, &h) != 0) { printf("create: %s\n", sg_last_error()); return 1; }
  float *dp, *dd;
  long long *di, *dm;
  cudaMalloc((void**)&dp, sizeof(pts));
  cudaMalloc((void**)&dd, sizeof(float) * N * K);
  cudaMalloc((void**)&di, sizeof(long long) * N * K);
  cudaMalloc((void**)&dm, sizeof(long long));
  cudaMemcpy(dp, pts, sizeof(pts), cudaMemcpyHostToDevice);
  int bad = 0;
  for (int prec = 0; prec <= 1; ++prec) {
    cudaMemset(dm, 0, sizeof(long long));
    int rc = sg_knn(h, dp, N, dp, N, D, LD, K, 0, 16, prec, (int64_t*)di, dd, (int64_t*)dm, NULL);
    if (rc != 0) { printf("knn: %s\n", sg_last_error()); return 1; }
    cudaDeviceSynchronize();
    static long long idx[N * K];
    static float dist[N * K];
    cudaMemcpy(idx, di, sizeof(idx), cudaMemcpyDeviceToHost);
    cudaMemcpy(dist, dd, sizeof(dist), cudaMemcpyDeviceToHost);
    for (int q = 0; q < N; ++q) {
      /* the k-th smallest distance to another point, brute force in double */
      double best[K];
      for (int j = 0; j < K; ++j) best[j] = 1e300;
      for (int r = 0; r < N; ++r) {
        if (r == q) continue;
        double acc = 0;
        for (int c = 0; c < D; ++c) { double t = (double)pts[q * LD + c] - pts[r * LD + c]; acc += t * t; }
        if (acc < best[K - 1]) {
          int j = K - 1;
          while (j > 0 && best[j - 1] > acc) { best[j] = best[j - 1]; --j; }
          best[j] = acc;
        }
      }
      for (int j = 0; j < K; ++j) {
        long long r = idx[q * K + j];
        if (r < 0 || r >= N || r == q) { bad++; continue; }
        double acc = 0;
        for (int c = 0; c < D; ++c) { double t = (double)pts[q * LD + c] - pts[r * LD + c]; acc += t * t; }
        if (acc > best[K - 1] * (1 + 1e-5) + 1e-6) bad++;
      }
    }
    printf("precision %d: %d wrong neighbours\n", prec, bad);
  }
  sg_destroy(h);
  return bad != 0;
}
"""


@pytest.mark.gpu
def test_c_program_runs_knn_on_the_gpu(tmp_path):
    """A C host allocates device memory with the CUDA runtime, calls sg_knn
    in both forms and checks every neighbour against brute force."""
    gcc = shutil.which("gcc")
    torch = pytest.importorskip("torch")
    if gcc is None or not torch.cuda.is_available():
        pytest.skip("needs gcc and a GPU")
    from scarf_gb300 import build
    lib = build.build()
    cu = build.cuda_lib_dir()
    inc = os.path.join(os.path.dirname(cu), "include")
    if not os.path.exists(os.path.join(inc, "cuda_runtime.h")):
        inc = os.path.join(os.path.dirname(os.path.dirname(build.nvcc())), "include")
    src = tmp_path / "knn.c"
    src.write_text(KNN_PROGRAM)
    exe = tmp_path / "knn"
    r = subprocess.run([gcc, "-std=c11", "-O2", str(src), "-I", os.path.join(ROOT, "include"), "-I", inc,
                        "-L", str(lib.parent), "-lscarfgpu", "-L", cu, "-lcudart", f"-Wl,-rpath,{lib.parent}",
                        f"-Wl,-rpath,{cu}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "precision 1: 0 wrong" in out.stdout
