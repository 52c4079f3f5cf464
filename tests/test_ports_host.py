"""Host side of the copper-port reduction (pcbqs_gb300.ports) against the reference's own outputs
(tests/golden/ports_strip.npz, made by make_ports_golden.py from pcbqs.mqs_ports): the single-frequency R/L
equivalent of the reference's port response, the drive of a response, and the input checks."""
import numpy as np
import pytest

from conftest import GOLDEN


def response():
    from pcbqs_gb300.ports import PortResponse
    with np.load(GOLDEN / 'ports_strip.npz') as d:
        g = {k: d[k] for k in d.files}
    return PortResponse(g['freqs'], [str(n) for n in g['ports']], g['Z_dc'], g['currents_dc']), g


def test_rl_equivalent_matches_reference():
    from pcbqs_gb300.ports import rl_equivalent, rl_error
    r, g = response()
    rl = rl_equivalent(r)
    assert rl['reference_Hz'] == float(g['rl_reference_Hz'])
    np.testing.assert_allclose(rl['R_ohm'], g['rl_R'], rtol=1e-12, atol=1e-18)
    np.testing.assert_allclose(rl['L_H'], g['rl_L'], rtol=1e-12, atol=1e-24)
    err = rl_error(rl, r)
    assert len(err) == len(r.frequencies) and err[-1] < 1e-9


def test_rl_equivalent_rejects_dc_and_non_passive():
    from pcbqs_gb300.ports import PortResponse, rl_equivalent
    r, _ = response()
    with pytest.raises(ValueError, match='positive reference frequency'):
        rl_equivalent(r, index=0)
    bad = PortResponse(np.array([1e6]), ['a', 'b'], np.array([[[1.0, 0], [0, -1.0]]], complex), np.zeros((1, 3, 2)))
    with pytest.raises(ValueError, match='non-passive'):
        rl_equivalent(bad)


def test_drive_is_the_weighted_sum_of_port_responses():
    r, _ = response()
    nf, _, npo = r.currents.shape
    a = np.arange(1, nf * npo + 1).reshape(nf, npo) * (1 + 0.5j)
    i = r.drive(a).i
    assert i.shape == (nf, r.currents.shape[1])
    np.testing.assert_allclose(i, (r.currents * a[:, None, :]).sum(-1), rtol=1e-14, atol=0)
    with pytest.raises(ValueError, match='amplitudes'):
        r.drive(np.ones((nf + 1, npo)))


def test_via_segments_of_the_via_pair():
    """The via pair's plated segments: read from the board, the branches they add (lower sheet's fan node to the
    upper one's, as MQS orders them), and their barrel resistance against the reference's via_resistance."""
    from pcbqs_gb300.board import Board
    from pcbqs_gb300.peec import via_resistance
    b = Board.load('viapair')
    assert b.nv == 2 and b.via_seg.shape == (2, 5)
    ends = b.via_ends()
    lower, upper = b.layer[[b.fans[f][0] for f in b.via_fans[:, 0]]], b.layer[[b.fans[f][0] for f in b.via_fans[:, 1]]]
    assert (lower == 0).all() and (upper == 1).all() and (ends[:, 0] != ends[:, 1]).all()
    with np.load(GOLDEN / 'ports_viapair.npz') as d:
        ref = d['via_R']
    np.testing.assert_allclose(via_resistance(b.via_seg, b.sigma, b.plating), ref, rtol=1e-14)
    assert Board.load('planes').nv == 0 and Board.load('planes').via_ends().shape == (0, 2)
