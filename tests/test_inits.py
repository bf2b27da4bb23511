import numpy as np

from formura_gb300 import inits


def test_splitmix64_known_answer():
    # First outputs of splitmix64 from state 0 (Vigna's reference implementation).
    z = inits.splitmix64(0, 3)
    assert [int(v) for v in z] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_inits_are_deterministic_and_in_range():
    a = inits.diffusion_2d(16, 32, seed=3)
    assert np.array_equal(a, inits.diffusion_2d(16, 32, seed=3))
    assert a.min() >= 0 and a.max() < 1
    U, V = inits.gray_scott_3d(32, 32, 32, seed=1)
    assert U.shape == (32, 32, 32)
    assert ((U == 1) | ((U > 0.49) & (U < 0.51))).all()
    assert ((V == 0) | ((V > 0.2474) & (V < 0.2526))).all()
    assert (V > 0).sum() > 0
