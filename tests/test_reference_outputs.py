"""The oracle against outputs of the reference's own code stored in
tests/golden/reference_outputs.npz (made by tests/golden/make_reference_outputs.py from the
reference's sources compiled against the VecCore stand-in). CPU only; needs no reference
tree. The GPU is compared with the same fixture in tests/test_gpu_reference_outputs.py."""
import os

import numpy as np
import pytest

from oracle.oracle import NAVSTATE_DTYPE, OracleGeometry
from reference_outputs import GEOMETRIES, SHAPES, fixture, geometry_inputs, shape_spec, oracle_geometry, shape_inputs
from vecgeom_gb300 import workloads as W

NT = os.cpu_count() or 1


@pytest.mark.parametrize("name", sorted(GEOMETRIES))
def test_oracle_transport_equals_reference_outputs(name):
    f = fixture()
    mod, fn, kw, n, seed, half, max_steps = GEOMETRIES[name]
    o = oracle_geometry(name)
    (x, y, z), (dx, dy, dz) = geometry_inputs(name)
    st, _ = o.locate(x, y, z, nthreads=NT)
    assert np.array_equal(st.view(np.uint8).reshape(n, 12), f[name + "/start"])
    ns, final, tr, trs, _ = o.transport(x, y, z, dx, dy, dz, st, max_steps, trace=True, nthreads=NT)
    mask = np.arange(max_steps)[None, :] < ns[:, None]
    assert np.array_equal(ns, f[name + "/nsteps"])
    assert np.array_equal(final.view(np.uint8).reshape(n, 12), f[name + "/final"])
    assert np.array_equal(tr[mask], f[name + "/trace_nav"])
    assert np.array_equal(trs[mask].view(np.uint64), f[name + "/trace_step"].view(np.uint64))
    assert ns.sum() > n


@pytest.mark.parametrize("name", SHAPES)
def test_oracle_shape_queries_equal_reference_outputs(name):
    f = fixture()
    o = OracleGeometry()
    sid = W.add_shape(o, *shape_spec(name))
    pts, dirs = shape_inputs(name)
    for q in range(6):
        d = dirs if q in (2, 3) else (None, None, None)
        got = np.asarray(o.shape_query(sid, q, *pts, *d, nthreads=NT))
        ref = f["%s/q%d" % (name, q)]
        if name == "torus2" and q in (2, 3):
            # the cubic resolvent calls the C library's cbrt/pow/cos/atan2, whose last bit can
            # differ between machines (the fixture was made on x86-64)
            assert np.all((got == ref) | (np.abs(got - ref) <= 1e-9 + 1e-12 * np.abs(ref))), q
        else:
            assert np.array_equal(got.view(np.uint8), ref.view(np.uint8)), q
