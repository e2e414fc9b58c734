"""Generate the golden fixtures under tests/golden/ (run in a container with scipy/mpmath).

* hankel.npz      H0^(1), H1^(1) at fixed arguments from scipy.special.hankel1 (AMOS, the
                  library the reference calls through complex_bessel) -- pins the oracle's and
                  the device's Hankel evaluators.
* known.npz       analytic / published values the reference's tests print:
                  circle single-layer eigenvalue (i pi/2) J_m(k) H_m^(1)(k)
                  (tests/ForwardMap/ComputeAx.cpp:69-70, here for k in {10, 20}, m = 3) and the
                  Helsing-Jiang open-line value u(0.17, 0.62)
                  (tests/ForwardMap/SolveAndPropagate.cpp:62).
* oracle_cfg1.npz oracle outputs for the unit circle, k = 10, 20 equal patches x 10 nodes
                  (N = 200): rectangular-polar matrix of patch 0, the direct forward map of the
                  mt19937(0) seeded density, so the oracle can be re-checked against itself.
"""
import os
import sys

import numpy as np
import scipy.special as sp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main():
    x = np.concatenate([np.logspace(-6, 5, 2001), np.linspace(2.5, 26.0, 1001),
                        np.array([1e-3, 0.5, 1.0, 2.999999, 3.0, 3.000001, 4.99, 5.0, 24.999999, 25.0, 25.000001, 1e4])])
    np.savez(os.path.join(HERE, "hankel.npz"), x=x, h0=sp.hankel1(0, x), h1=sp.hankel1(1, x))
    lam = {f"circle_eig_k{int(k)}_m3": 1j * np.pi / 2 * sp.jv(3, k) * sp.hankel1(3, k) for k in (10.0, 20.0)}
    np.savez(os.path.join(HERE, "known.npz"), helsing_jiang=np.complex128(0.02788626934981090 - 0.75932847390327920j), **lam)
    from oracle import oracle as O
    O.build()
    fm = O.OracleForwardMap([O.curve_circle()], 10, 0.01, 1.0, 10.0, patches_per_curve=20)
    fm.precompute(10.0)
    d = O.seeded_density(fm.N)
    np.savez(os.path.join(HERE, "oracle_cfg1.npz"), precomp0=fm.precomp_matrix(0), density=d,
             y_direct=fm.compute_Ax_unacc(d))
    print("wrote golden fixtures to", HERE)


if __name__ == "__main__":
    main()
