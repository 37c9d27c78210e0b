"""The boundary is plain C: a C99 program that includes include/mhdgb.h, links libmhdgb.so and
calls it with no Python in between.  On the CPU the program compiles and links with gcc (the
header is valid C) and reports the library's validation; with a GPU it also creates a problem,
sets the Taylor-Green velocity, steps it and reads the diagnostics."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include "mhdgb.h"

int main(int argc, char** argv) {
  int run = argc > 1;
  mhd_params p = {0};
  p.n = 17; p.L = 6.283185307179586; p.nu = 1e-2; p.eta = 1e-2; p.dt = 1e-3; p.scheme = MHD_RK4;
  mhd_handle h = NULL;
  if (mhd_create(&p, &h) != MHD_ERR_INVALID) { printf("expected invalid n\n"); return 1; }
  printf("validation: %s\n", mhd_last_error());
  int kx, kp, kn;
  if (mhd_kept_modes(32, &kx, &kp, &kn) || kx != 10 || kp != 10 || kn != 10) return 2;
  if (!run) return 0;
  p.n = 32;
  if (mhd_create(&p, &h)) { printf("create: %s\n", mhd_last_error()); return 3; }
  const int n = 32;
  float* f = (float*)malloc(sizeof(float) * n * n * n);
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double x = -M_PI + 2 * M_PI * i / n, y = -M_PI + 2 * M_PI * j / n, z = -M_PI + 2 * M_PI * k / n;
        f[(k * n + j) * n + i] = (float)(sin(x) * cos(y) * cos(z));
      }
  if (mhd_set_physical(h, 0, f)) return 4;  /* u = (sin x cos y cos z, -cos x sin y cos z, 0), B = 0 */
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double x = -M_PI + 2 * M_PI * i / n, y = -M_PI + 2 * M_PI * j / n, z = -M_PI + 2 * M_PI * k / n;
        f[(k * n + j) * n + i] = (float)(-cos(x) * sin(y) * cos(z));
      }
  if (mhd_set_physical(h, 1, f)) return 4;
  double d0[8], d1[8];
  if (mhd_diagnostics(h, d0, 8) || mhd_step(h, 10) || mhd_diagnostics(h, d1, 8)) {
    printf("step: %s\n", mhd_last_error());
    return 5;
  }
  printf("E_u %.9g -> %.9g, t %.6g\n", d0[0], d1[0], d1[7]);
  mhd_destroy(h);
  free(f);
  return (d1[0] < d0[0] && d1[0] > 0.9 * d0[0] && fabs(d1[7] - 0.01) < 1e-6) ? 0 : 6;
}
"""


def _build(tmp_path, pkg):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    lib = pkg._lib.load()._name
    src = tmp_path / "abi.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "abi"
    cmd = [gcc, "-std=c99", "-O1", "-Wall", "-Werror", "-D_DEFAULT_SOURCE", "-I", os.path.join(ROOT, "include"),
           str(src), lib, "-Wl,-rpath," + os.path.dirname(lib), "-lm", "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def test_c_program_builds_and_validates(tmp_path, pkg):
    exe = _build(tmp_path, pkg)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "unsupported grid size" in res.stdout


@pytest.mark.gpu
def test_c_program_steps_on_the_gpu(tmp_path, pkg):
    exe = _build(tmp_path, pkg)
    res = subprocess.run([str(exe), "run"], capture_output=True, text=True, timeout=300)
    print(res.stdout)
    assert res.returncode == 0, res.stdout + res.stderr
