"""xoshiro256** and its seedings against the reference's known answers
(crates/caroli-disorder/src/rng.rs:87-105, values printed by gfortran 16)."""
from caroli_gb300.disorder import Moments, Xoshiro256, choose_sites


def test_reproduces_gfortran():
    r = Xoshiro256.gfortran(12345)
    expected = [4.65636743897908767e-01, 1.00833111555351462e-01, 8.41914420882911130e-01,
                7.73831493534653414e-01, 1.80372332904081167e-01, 8.44873831312145440e-01]
    assert [r.uniform() for _ in expected] == expected
    assert Xoshiro256.gfortran(1237).uniform() == 4.72208155982870581e-01
    assert Xoshiro256.gfortran_put([1, 2, 3, 4, 5, 6, 7, 8]).uniform() == 4.71070899360821249e-01


def test_seeds_differ_and_range():
    a = Xoshiro256.seed_from_u64(1).uniforms(4)
    b = Xoshiro256.seed_from_u64(2).uniforms(4)
    assert list(a) != list(b)
    assert all(0.0 <= x < 1.0 for x in a)


def test_choose_sites_distinct():
    r = Xoshiro256.seed_from_u64(7)
    picked = choose_sites(r, list(range(100)), 40)
    assert len(set(picked)) == 40


def test_polarized_moments_are_z():
    r = Xoshiro256.seed_from_u64(3)
    for m in Moments.polarized(1.0).draw(r, 10):
        assert m[2] == 1.0 and abs(m[0]) == 0.0 and abs(m[1]) == 0.0
