"""The transport oracle (oracle/transport.py) pinned against the advection oracle: with every
element active and a constant depth h, c h evolves as h times the advected concentration, so the
transport of the 'rotation' discs must equal the advection of c = c h / h by the same velocity
(to roundoff: the transport keeps hatM = I where the advection integrates hatM)."""
import numpy as np

from oracle import advection as ADV
from oracle import transport as TR


def test_unmasked_transport_equals_advection():
    kw = dict(hmax=2 ** -3, numSteps=8, tEnd=8 * 0.01, p=1)
    t = TR.main(isMask=False, numSpecies=1, **kw)
    a = ADV.Struct(dict(testcase='solid_body', isSlopeLim=True, typeSlopeLim='linear', ordRK=2, **kw))
    a.problemName = 'advection'
    ADV.configureProblem(a)
    r = 0.0225 / np.sqrt(2)
    a.c0Cont = lambda x1, x2: ((((x1 - 0.5) ** 2 + (x2 - 0.75) ** 2 <= r) * 1.0
                                + ((x1 - 0.25) ** 2 + (x2 - 0.5) ** 2 <= r)
                                + ((x1 - 0.5) ** 2 + (x2 - 0.25) ** 2 <= r)
                                + ((x1 - 0.75) ** 2 + (x2 - 0.5) ** 2 <= r)))
    ADV.preprocessProblem(a)
    ADV.initializeProblem(a)
    ADV.run_loop(a)
    rel = np.linalg.norm(t.concDisc[0] - a.cDisc) / np.linalg.norm(a.cDisc)
    assert rel < 1e-12, rel
    assert np.allclose(t.cDisc[0], 0.1 * t.concDisc[0], rtol=1e-12, atol=1e-15)


def test_masks_follow_the_discs():
    t = TR.main(hmax=2 ** -4, numSteps=4, tEnd=4 * 0.01, numSpecies=2)
    for s in range(2):
        m = t.mask[s]
        assert 0 < m.sum() < m.size            # the discs, not the whole square
        assert np.abs(t.concDisc[s][~m, 0]).max() < 1e-6 * (s + 1) * 10
