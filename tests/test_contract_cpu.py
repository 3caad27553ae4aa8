"""The generated element-row code of the order-1/2 assembly kernel
(sucem-fem_gb300/csrc/n1curl_contract.h), compiled for the host with g++
and evaluated in double precision on random tetrahedra, against the
oracle's element matrices (an independent, sympy-exact derivation of the
same reference tensors).  Covers every (order, edge/face, local index) and
both the fused (S + T part) and split (S, T apart) forms; the split form is
also run in single precision, whose compensated sums must stay exact to
~1e-13 of the size of their terms where those terms cancel."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import fem

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(HERE), "sucem-fem_gb300", "csrc", "n1curl_contract.h")

DRIVER = r"""
#include <cmath>
#include <cstdio>
using std::fma;
#define __device__
#define __forceinline__ inline
#include "%s"
using namespace sucem::contract;
using std::fmaf;
template <int O, bool F, int LE>
void rows(const double* g, const float* gf) {
  Rows<O, F, LE>::fused(g, [&](int j, int b, double v) { std::printf("f %%d %%d %%d %%d %%d %%.17g\n", O, F, LE, j, b, v); });
  Rows<O, F, LE>::split(g, [&](int j, int b, const Dot2<double>& s, const Dot2<double>& t) {
    std::printf("s %%d %%d %%d %%d %%d %%.17g %%.17g\n", O, F, LE, j, b, s.s, t.s);
  });
  // single precision: the unrounded double-float sums s + c
  Rows<O, F, LE>::split(gf, [&](int j, int b, const Dot2<float>& s, const Dot2<float>& t) {
    std::printf("t %%d %%d %%d %%d %%d %%.17g %%.17g\n", O, F, LE, j, b, (double)s.s + (double)s.c,
                (double)t.s + (double)t.c);
  });
}
int main() {
  double g[12];
  float gf[24];  // single precision: the coefficients as float hi + lo
  for (int i = 0; i < 12; ++i) {
    if (std::scanf("%%lf", &g[i]) != 1) return 1;
    gf[i] = (float)g[i];
    gf[i + 12] = (float)(g[i] - (double)gf[i]);
  }
  rows<1, false, 0>(g, gf); rows<1, false, 1>(g, gf); rows<1, false, 2>(g, gf);
  rows<1, false, 3>(g, gf); rows<1, false, 4>(g, gf); rows<1, false, 5>(g, gf);
  rows<2, false, 0>(g, gf); rows<2, false, 1>(g, gf); rows<2, false, 2>(g, gf);
  rows<2, false, 3>(g, gf); rows<2, false, 4>(g, gf); rows<2, false, 5>(g, gf);
  rows<2, true, 0>(g, gf); rows<2, true, 1>(g, gf); rows<2, true, 2>(g, gf);
  rows<2, true, 3>(g, gf);
  return 0;
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("contract")
    src = d / "drv.cpp"
    src.write_text(DRIVER % HEADER)
    exe = d / "drv"
    subprocess.run([gxx, "-O1", "-std=c++17", "-ffp-contract=off", "-o", str(exe), str(src)],
                   check=True)
    return str(exe)


def _metrics(coords, cells):
    J, det, Jinv = fem.geometry(coords, cells)
    adet = abs(det[0])
    Gs = J[0].T @ J[0] / adet
    Gt = Jinv[0] @ Jinv[0].T * adet
    sym = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    return np.array([Gs[p, q] for p, q in sym] + [Gt[p, q] for p, q in sym])


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_generated_rows_match_oracle(driver, seed):
    rng = np.random.default_rng(seed)
    coords = rng.standard_normal((4, 3))
    cells = np.array([[0, 1, 2, 3]])
    g = _metrics(coords, cells)
    out = subprocess.run([driver], input=" ".join("%.17g" % x for x in g), capture_output=True,
                         text=True, check=True).stdout.split("\n")
    ref = {o: fem.element_matrices(coords, cells, o, [1.0], [1.0]) for o in (1, 2)}
    # exact element rows and the size of their terms
    from oracle import n1curl_exact
    exact, termsum = {}, {}
    for o in (1, 2):
        R = n1curl_exact.reference_tensors(o)
        Kc, Km = fem._sym6(R["curl"]), fem._sym6(R["mass"])
        exact[o] = (np.einsum("m,mab->ab", g[:6], Kc), np.einsum("m,mab->ab", g[6:], Km))
        termsum[o] = (np.einsum("m,mab->ab", np.abs(g[:6]), np.abs(Kc)),
                      np.einsum("m,mab->ab", np.abs(g[6:]), np.abs(Km)))
    seen = 0
    for line in out:
        if not line:
            continue
        parts = line.split()
        kind, o, face, le, j, b = parts[0], *map(int, parts[1:6])
        a = 12 + 2 * le + j if face else o * le + j
        S, T = ref[o][0][0], ref[o][1][0]
        scale = max(np.abs(S).max(), np.abs(T).max())
        if kind == "f":
            assert abs(float(parts[6]) - (S[a, b] + T[a, b])) <= 1e-13 * scale
        elif kind == "t":
            # compensated single-precision sums (coefficients and constants
            # as float hi + lo, result kept as s + c): exact to ~1e-13 of the
            # size of their terms, even where the terms cancel
            for q in (0, 1):
                e = exact[o][q][a, b]
                assert abs(float(parts[6 + q]) - e) <= 1e-12 * termsum[o][q][a, b] + 1e-15 * scale
        else:
            assert abs(float(parts[6]) - S[a, b]) <= 1e-13 * scale
            assert abs(float(parts[7]) - T[a, b]) <= 1e-13 * scale
        seen += 1
    # split forms (double and float): every entry of every local entity's rows
    assert seen >= 2 * (6 * 6 + 10 * 2 * 20) + 6 * 6
