"""Golden copper-port reductions from the reference's own CopperPorts (magnetic MQS, no capacitance).

    PCBQS_REFERENCE_SRC=<checkout>/src python tests/golden/make_ports_golden.py     (this container only: needs the reference checkout)

The model object is the one make_peec_golden.py builds around a given mesh (src/pcbqs/mqs.py:300-420), with
capacitance off, so that pcbqs.mqs_ports.CopperPorts (src/pcbqs/mqs_ports.py:27-53) reduces the copper to its
current ports by the reference's dense direct solve (direct_ports, :56-69). Only boards whose ports join terminals of
one connected net qualify (the strip: p1 left->mid, p2 mid->right; the via pair: its loop through two plated vias).

Writes tests/golden/ports_<board>.npz: freqs (DC included), port names, Z (nf, np, np) and branch currents
(nf, nbranch, np) for conductor_loss 'dc' and 'slab', and the reference's rl_equivalent of the 'dc' response at its
highest frequency (R_ohm, L_H); for a board with plated vias (the via pair) also the reference's via_resistance and
via_inductance of its segments (src/pcbqs/mqs.py:132-153).

    PCBQS_REFERENCE_SRC=<checkout>/src python tests/golden/make_ports_golden.py [strip|viapair]
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parents[1]))

from make_peec_golden import reference_model  # noqa: E402


def main(name='strip'):
    from pcbqs_gb300.board import Board
    b = Board.load(name)
    freqs = np.array([0.0, 1e5, 1e6, 1e7])
    out = dict(freqs=freqs)
    for loss in ('dc', 'slab'):
        q = reference_model(b, loss)
        q.capacitance = False
        from pcbqs.mqs_ports import CopperPorts, rl_equivalent
        r = CopperPorts(q).extract(freqs)
        out['ports'] = np.array(r.names)
        out[f'Z_{loss}'] = r.impedance
        out[f'currents_{loss}'] = r.currents
        if loss == 'dc':
            rl = rl_equivalent(r)
            out['rl_R'], out['rl_L'] = np.array(rl['R_ohm']), np.array(rl['L_H'])
            out['rl_reference_Hz'] = rl['reference_Hz']
        print(name, loss, 'loops', q._assemble()['C'].shape, np.round(r.impedance[2], 9))
    if b.nv:
        from pcbqs.mqs import via_inductance, via_resistance
        out['via_R'] = via_resistance(q.vseg, q.sigma, q.plating)
        out['via_L'] = via_inductance(q.vseg)
        # the field of the last ('slab') response driven 1 A per port, sheets and vias, at 1 MHz, from the
        # reference's MQS.h_field, on a line of points 0.5 mm over the upper strip and beside the vias
        res = r.drive(np.ones((len(freqs), len(r.names))))
        xs = np.linspace(-1e-3, 11e-3, 25)
        pts = np.r_[np.c_[xs, np.full(25, 1e-3), np.full(25, 0.7e-3)], np.c_[np.full(5, 9e-3), np.full(5, 1e-3),
                                                                             np.linspace(0.02e-3, 0.18e-3, 5)]]
        out['field_pts'], out['field_fi'] = pts, 2
        out['field_H'] = q.h_field(res, 2, pts)
    np.savez_compressed(HERE / f'ports_{name}.npz', **out)


if __name__ == '__main__':
    main(*sys.argv[1:2])
