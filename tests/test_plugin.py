"""Registration of the cuda solvers into the reference's own factory (drop-in),
checked in-process against the live reference where it is importable."""
import numpy as np
import pytest

import problems
import pysit_gb300 as api

pysit_live = pytest.importorskip("pysit_live")
if not pysit_live.available():
    pytest.skip("reference tree not present on this host", allow_module_level=True)


@pytest.fixture(scope="module")
def pysit():
    p = pysit_live.import_pysit()
    from pysit_gb300 import plugin
    plugin.register(p)
    return p


@pytest.mark.parametrize("name,dim", [("1d", 1), ("o6", 2), ("3d", 3)])
@pytest.mark.parametrize("order", [2, 4, 6, 8])
def test_reference_factory_resolves_cuda(pysit, name, dim, order):
    """As pysit/solvers/tests/test_factories.py:55-79 does for 'cpp'."""
    m, *_ = problems.build(pysit, name, kernel="cpp")
    s = pysit.ConstantDensityAcousticWave(m, spatial_accuracy_order=order, kernel_implementation="cuda")
    assert type(s).__name__ == f"ConstantDensityAcousticTimeScalar_{dim}D_cuda"
    assert s.supports["kernel_implementation"] == "cuda"
    s._plans["key"] = object()
    s.release_plans()
    assert s._plans == {}
    # the cpp solver is still selected for 'cpp'
    c = pysit.ConstantDensityAcousticWave(m, spatial_accuracy_order=order, kernel_implementation="cpp")
    assert type(c).__name__ == f"ConstantDensityAcousticTimeScalar_{dim}D_cpp"


def test_registration_is_idempotent(pysit):
    from pysit_gb300 import plugin
    a = plugin.register(pysit)
    b = plugin.register(pysit)
    assert a == b


@pytest.mark.parametrize("name", ["cfg1", "o8", "3d"])
def test_reference_shot_adapter_matches_mirror_taps(pysit, name):
    from pysit_gb300.plugin import ReferenceShotAdapter
    rm, rshots, *_ = problems.build(pysit, name, kernel="cpp")
    mm, mshots, *_ = problems.build(api, name)
    a = ReferenceShotAdapter(rshots[0], rm)
    c1, p1, w1 = a.sources.taps()
    c2, p2, w2 = mshots[0].sources.taps()
    o1, o2 = np.argsort(c1), np.argsort(c2)
    np.testing.assert_array_equal(c1[o1], c2[o2])
    np.testing.assert_allclose(w1[o1], w2[o2], rtol=1e-15)
    rc1, rr1, ws1, wi1 = a.receivers.taps()
    rc2, rr2, ws2, wi2 = mshots[0].receivers.taps()
    o1, o2 = np.lexsort((rc1, rr1)), np.lexsort((rc2, rr2))
    np.testing.assert_array_equal(rc1[o1], rc2[o2])
    np.testing.assert_array_equal(rr1[o1], rr2[o2])
    np.testing.assert_allclose(ws1[o1], ws2[o2], rtol=1e-15)
    np.testing.assert_allclose(wi1[o1], wi2[o2], rtol=1e-15)
    ts = np.arange(50) * 1e-3
    np.testing.assert_allclose(a.sources.amplitudes(ts), mshots[0].sources.amplitudes(ts), rtol=1e-15)
