"""Hype on the CPU: the hyperboloid ring builds identically in the product and the oracle
(NavIndex tables, BVHs, extents), and the product's extents equal the oracle's for every
variant (hollow, solid, cylindrical and conical inner surface)."""
import numpy as np
import pytest

import vecgeom_gb300 as vg
from oracle.oracle import OracleGeometry
from test_cpu_build import compare_builders
from vecgeom_gb300 import workloads as W


@pytest.mark.parametrize("name", sorted(W.HYPES))
def test_extents_match_oracle(name):
    g, o = vg.Geometry(), OracleGeometry()
    a = np.array(g.shape_extent(g.add_hype(*W.HYPES[name])))
    b = np.array(o.shape_extent(o.add_hype(*W.HYPES[name])))
    assert np.array_equal(a, b)


def test_hype_ring_builds_identically():
    compare_builders(W.build_hype_ring)
