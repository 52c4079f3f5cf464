"""The layered-dielectric host side against the reference's own fixtures: the image series of the static ray
expansion (src/pcbqs/electrostatic.py:82-148) against the reference's spectral transmission-line fixture (the check
of tests/test_electrostatic.py:12-19) and the reference's image lists and spline arguments for the tiny board."""
import numpy as np
import pytest

from conftest import GOLDEN
from pcbqs_gb300.fill import EPS0
from pcbqs_gb300.layered import DielectricStack, spline_arguments


def fixture(name):
    with np.load(GOLDEN / f'layered_{name}.npz') as d:
        return {k: d[k] for k in d.files}


@pytest.mark.parametrize('o,s', [(0, 0), (0, 3), (1, 2), (2, 2), (3, 1)])
def test_images_match_static_limit_of_spectral_network(o, s):
    data = fixture('spectral')
    images = DielectricStack(data['z'], data['eps'], tol=1e-10)
    k = data['k']
    transform = sum(c * np.exp(-k * d) for d, c in images.images(s, o)) / (2 * EPS0 * k)
    assert transform == pytest.approx(data[f'r{o}_{s}'], rel=3e-8)


def test_image_lists_and_spline_match_reference():
    g = fixture('tiny')
    z0, z1, er, tand = g['slab']
    stack = DielectricStack.slab(z0, z1, er, tand)
    for o, s in g['pairs']:
        images = stack.images(int(s), int(o))
        d = np.array([x for x, _ in images])
        c = np.array([y for _, y in images])
        assert np.array_equal(d, g[f'images_{o}_{s}_d'])
        assert np.array_equal(c, g[f'images_{o}_{s}_c'])
        dd, cc, sx, sc = spline_arguments(images, float(g['rho_max']), 3.0)
        assert np.array_equal(dd, d) and np.array_equal(cc, c)
        assert sx == pytest.approx(g[f'spline_{o}_{s}_x'], rel=1e-15, abs=0)
        assert sc == pytest.approx(g[f'spline_{o}_{s}_c'], rel=1e-12, abs=1e-12 * np.abs(sc).max())


def test_stack_validation():
    with pytest.raises(ValueError):
        DielectricStack([0.0, 0.0], [1, 4, 1])
    with pytest.raises(ValueError):
        DielectricStack([0.0, 1e-3], [1, 4 + 1j, 1])          # active medium
    stack = DielectricStack.slab(0, 2e-4, 4.3)
    with pytest.raises(ValueError, match='interface'):
        stack.interface(1e-4)
    assert stack.images(0, 0)[0][0] == 0.0                      # the direct term first
