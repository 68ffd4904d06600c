"""The reference arm's extrapolation of the two workloads too large to time on host cores.

C2 (cube(64) [P2,P2,P2]) and C3 (cube(160) P1) are timed at four smaller sizes of the same varf
and extrapolated: nnz as the exact cubic through the four sizes, assembly linear in the
elements, CG iterations linear in n, time per iteration linear in nnz.  The entry counts used
here are the ones the oracle produces at those sizes (FreeFEM's patterns); the cubic must give
the full-size counts the device assembles (547 739 145 and 61 979 041), and on data that is
exactly linear the extrapolated time must be the formula's value."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
import bench  # noqa: E402

NNZ = {
    "elasticity_p2_cube64": ({6: 493137, 8: 1141065, 10: 2196369, 12: 3758409}, 547739145),
    "diffusion_p1_cube160": ({16: 66961, 24: 219673, 32: 513313, 40: 993961}, 61979041),
}


def _runs(cfgname, a=2e-8, b=1e-3, c=5.5, d=30.0, e=3e-9, f=2e-6):
    """Synthetic oracle timings, exactly linear in the fitted variables, two runs per size."""
    kind = bench.CONFIGS[cfgname]["mesh"][0]
    out = []
    for n, nnz in NNZ[cfgname][0].items():
        nt = 6 * n ** 3
        its = c * n + d
        for _ in range(2):
            out.append({"size": (kind, n), "nt": nt, "nnz": nnz, "ndof": 0, "t_asm": a * nt + b,
                        "t_cg": its * (e * nnz + f), "its": its})
    return out


@pytest.mark.parametrize("cfgname", sorted(NNZ))
def test_extrapolation_reproduces_full_size_nnz_and_linear_model(cfgname):
    a, b, c, d, e, f = 2e-8, 1e-3, 5.5, 30.0, 3e-9, 2e-6
    t, fit = bench.ref_extrapolated(cfgname, _runs(cfgname, a, b, c, d, e, f))
    N = bench.CONFIGS[cfgname]["mesh"][1]
    assert fit["nnz_full"] == NNZ[cfgname][1]
    assert fit["sizes"] == sorted(NNZ[cfgname][0])
    its = c * N + d
    expect = a * 6 * N ** 3 + b + its * (e * NNZ[cfgname][1] + f)
    assert abs(fit["cg_iterations_full"] - its) <= 1e-9 * its
    assert abs(t - expect) <= 1e-6 * expect
