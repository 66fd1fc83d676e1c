"""The CUDA shape kernels against the known answers of the reference's own unit tests
(tests/golden/unit_*.json) and against the oracle on the same points: every hard assert
passes, soft checks pass except the documented exceptions, and results equal the oracle's
(Inside exactly; distances and safeties within 1e-9 mm + 1e-12 relative, every shape
including Torus2)."""
import numpy as np
import pytest

import golden_util as G
from conftest import dist_mismatch

pytestmark = pytest.mark.gpu


def _run(torch, g, pv, qi, p, d):
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0")
    x, y, z = dev(p[:, 0]), dev(p[:, 1]), dev(p[:, 2])
    n = len(p)
    if qi == 0:
        out = torch.empty(n, dtype=torch.int32, device="cuda:0")
        g.inside(pv, x, y, z, out)
    elif qi == 1:
        out = torch.empty(n, dtype=torch.uint8, device="cuda:0")
        g.contains(pv, x, y, z, out)
    elif qi in (2, 3):
        out = torch.empty(n, dtype=torch.float64, device="cuda:0")
        f = g.distance_to_in if qi == 2 else g.distance_to_out
        f(pv, x, y, z, dev(d[:, 0]), dev(d[:, 1]), dev(d[:, 2]), out)
    else:
        out = torch.empty(n, dtype=torch.float64, device="cuda:0")
        (g.safety_to_in if qi == 4 else g.safety_to_out)(pv, x, y, z, out)
    return out.cpu().numpy()


@pytest.mark.parametrize("name", G.FILES)
def test_kernels_match_reference_unit_tests(cuda, name):
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    doc = G.load(name)
    fails, diff = [], []
    for shape, q, cs, p, d in G.grouped(doc):
        spec = doc["shapes"][shape]
        g, o = vg.Geometry(), OracleGeometry()
        pv, opv = G.build(g, spec), G.build(o, spec)
        qi = G.QUERY_ID[q]
        got = _run(cuda, g, pv, qi, p, d)
        cols = [p[:, k].copy() for k in range(3)] + ([d[:, k].copy() for k in range(3)] if qi in (2, 3) else [])
        ref, _ = o.query(opv, qi, *cols)
        for c, v in zip(cs, got):
            if not G.case_passes(name, c, v):
                fails.append((c["line"], shape, q, c["expected"], float(v)))
        if qi in (0, 1):
            bad = got.astype(np.int64) != ref.astype(np.int64)
        else:
            bad = dist_mismatch(got, ref)
        diff += [(shape, q, float(a), float(b)) for a, b in zip(got[bad], ref[bad])]
    assert not fails, fails[:5]
    assert not diff, diff[:5]
