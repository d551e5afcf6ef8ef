"""The forward-mode dual numbers the discrete adjoint differentiates the
per-cell property chain with (ressim_gb300/csrc/dual.cuh), compiled for the
host with g++ (the CUDA qualifiers defined away): values, partial
derivatives of rational expressions, mixed double/dual operators, compound
assignment, constant-exponent powers and comparisons against closed forms."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#define __host__
#define __device__
#include <math.h>  // ::isnan and ::pow in the global namespace, as CUDA provides them
#include <cstdio>
#include "dual.cuh"
using D = rsg::Dual<2>;
int main() {
  const double xs[3][2] = {{1.5, -0.25}, {0.3, 2.0}, {-4.0, 0.75}};
  for (auto& xy : xs) {
    D x = D::var(xy[0], 0), y = D::var(xy[1], 1);
    D f = (x * y + 3.0) / (x - y);       // rational
    D g = 2.0 - x / (1.0 + y * y);       // mixed double on both sides
    D h = x;
    h *= y; h += 1.0; h /= (y + 5.0); h -= x; // compound forms
    D p = rsg::dual_pow(x * x + 1.0, 2.5);
    printf("%.17g %.17g %.17g\n", f.v, f.d[0], f.d[1]);
    printf("%.17g %.17g %.17g\n", g.v, g.d[0], g.d[1]);
    printf("%.17g %.17g %.17g\n", h.v, h.d[0], h.d[1]);
    printf("%.17g %.17g %.17g\n", p.v, p.d[0], p.d[1]);
    printf("%d %d %d %g\n", (int)(x < y), (int)(x >= 0.3), (int)(1.0 == x), rsg::val(-x));
  }
  return 0;
}
"""


def _closed_forms(x, y):
    f = (x * y + 3) / (x - y)
    fx = (y * (x - y) - (x * y + 3)) / (x - y) ** 2
    fy = (x * (x - y) + (x * y + 3)) / (x - y) ** 2
    g = 2 - x / (1 + y * y)
    gx, gy = -1 / (1 + y * y), 2 * x * y / (1 + y * y) ** 2
    h = (x * y + 1) / (y + 5) - x
    hx = y / (y + 5) - 1
    hy = (x * (y + 5) - (x * y + 1)) / (y + 5) ** 2
    u = x * x + 1
    p, px = u ** 2.5, 2.5 * u ** 1.5 * 2 * x
    return [(f, fx, fy), (g, gx, gy), (h, hx, hy), (p, px, 0.0)]


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_dual_algebra(tmp_path):
    src = tmp_path / "dual_test.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "dual_test"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "ressim_gb300", "csrc"), str(src), "-o",
                    str(exe)], check=True)
    lines = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines()
    assert len(lines) == 15
    for i, (x, y) in enumerate([(1.5, -0.25), (0.3, 2.0), (-4.0, 0.75)]):
        block = lines[5 * i:5 * i + 5]
        for row, want in zip(block[:4], _closed_forms(x, y)):
            got = np.array([float(t) for t in row.split()])
            assert np.allclose(got, want, rtol=1e-13, atol=1e-15), (row, want)
        lt, ge, eq, neg = block[4].split()
        assert (int(lt), int(ge), int(eq)) == (int(x < y), int(x >= 0.3), int(x == 1.0))
        assert float(neg) == -x
