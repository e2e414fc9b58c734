"""Generate tests/golden/oracle_kite_k8000.npz: the oracle at the largest benchmark kite.

The kite (x = cos t + 0.65 cos 2t - 0.65, y = 1.5 sin t) at k = 8000, 8192 equal patches x 16
Fejer nodes (N = 131072), combined field with eta = k, IFGF 5 x 5 cones on the deepest tree the
neighbourhood check accepts (10 levels).  The oracle's IFGF takes minutes on one core at this
size, too long for the test suite, so its outputs on 1024 sampled rows (four ranges of 256
rows spread over the curve) are stored here for the seeded density of std::mt19937(0):

* rows      the sampled point indices (patch order)
* far_ifgf  BoxTree::Solve (IFGF_Source/BoxTree.h:1020-1071) of the quadrature-weighted
            density, with the exclusion sets of ForwardMap.tpp:567-607
* far_sum   the exclusion-matched O(N^2) sum of the same intensities
            (tests/IFGF/IgnoreSingNSing.cpp:65-117)
* acc       compute_Ax_acc (ForwardMap.tpp:609-655): singular correction + IFGF far field +
            the jump term of the combined field
* nlevels   the tree depth

Run from the repository root: python tests/golden/make_golden_kite.py (about four minutes).
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

K = 8000.0
PATCHES = 8192
NLEVELS = 10


def sample_rows(n, count=1024, pieces=4):
    step = count // pieces
    return [(n * j // pieces, n * j // pieces + step) for j in range(pieces)]


def main():
    from oracle import oracle as O
    O.build()
    t0 = time.time()
    om = O.OracleForwardMap([O.curve_kite()], 16, 0.01, 1.0, K, patches_per_curve=PATCHES, formulation="combined")
    om.precompute(K)
    om.setup_ifgf(K, NLEVELS)
    d = O.seeded_density(om.N)
    rho = d * om.point_weights()[0]
    ranges = sample_rows(om.N)
    rows = np.concatenate([np.arange(r0, r1) for r0, r1 in ranges])
    far_ifgf = om.ifgf_far(rho)[rows]
    far_sum = np.concatenate([om.direct_excluded(rho, r) for r in ranges])
    acc = om.compute_Ax_acc(d)[rows]
    np.savez(os.path.join(HERE, "oracle_kite_k8000.npz"), rows=rows, far_ifgf=far_ifgf, far_sum=far_sum, acc=acc,
             nlevels=np.int64(NLEVELS), k=np.float64(K), patches=np.int64(PATCHES))
    print(f"wrote oracle_kite_k8000.npz in {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
