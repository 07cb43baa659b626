"""Cross-method check of the oracle: nested dissection (oracle/nested_oracle.cpp) against the
recursive Green's function (oracle/rgf.py) on the same systems and self-energies, as the
reference checks its two methods against each other (tests/nested.rs:42-50, cubic :160-177)."""
import numpy as np
import pytest

from systems import bench_system, clean_bhz_ribbon, cubic_wire, graphene_ribbons, magnetic_bhz, oracle_T


def _rgf(sys_, sigma, config=0):
    from oracle import rgf

    return rgf.transmission(sys_.system, sigma.energy, sigma.blocks, config)


@pytest.mark.parametrize("make, energies", [
    (lambda: clean_bhz_ribbon(16, 10), (-0.05, 0.0, 0.05, 0.2)),
    (lambda: magnetic_bhz(20, 12, configs=2), (-0.12, 0.03)),
    (lambda: bench_system("square-anderson", 16), (-1.2, 0.3)),
    (lambda: graphene_ribbons(1)[0], (-0.4, 0.2)),
    (lambda: cubic_wire(8, 4, 4), (-0.5, 0.4)),
])
def test_nested_dissection_matches_rgf(make, energies):
    sys_ = make()
    for e in energies:
        s = sys_.self_energies(e)
        for c in range(sys_.config_count()):
            nd = oracle_T(sys_, s, config=c)
            rg = _rgf(sys_, s, config=c)
            assert abs(nd - rg) <= 1e-9 * (1 + abs(rg)), (e, c, nd, rg)
