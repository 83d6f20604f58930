"""Engine self-tests on the GPU: the correctly rounded division by 3 of the eikonal
update equals the IEEE quotient x / 3.0f for every non-NaN float input, the branch-free and
packed forms of the reference's Godunov update equal its branching form, and the x sweep's
TMA tiles land where its swizzled indexing reads them."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def test_div3_exhaustive(engine):
    from gbsdf import _lib

    L = _lib.load()
    res = C.c_uint64(123)
    err = C.create_string_buffer(256)
    rc = L.gbsdf_selftest(0, 0, C.byref(res), err, len(err))
    assert rc == 0, err.value
    assert res.value == 0, f"{res.value} inputs round differently"


def test_godunov_forms_agree(engine):
    """godunov_ref_nb, godunov_ref_nbp and both lanes of godunov_ref_pair against the
    reference's branching update on 2^30 generated neighbour triples."""
    from gbsdf import _lib

    L = _lib.load()
    res = C.c_uint64(123)
    err = C.create_string_buffer(256)
    rc = L.gbsdf_selftest(2, 0, C.byref(res), err, len(err))
    assert rc == 0, err.value
    assert res.value == 0, f"{res.value} updates differ from the reference's branching form"


def test_tma_tile_layout(engine):
    """The x sweep's TMA tile: every element of five boxes (inside, across the lattice's
    low and high faces) is where the swizzled index says, with NaN outside the lattice."""
    from gbsdf import _lib

    L = _lib.load()
    res = C.c_uint64(123)
    err = C.create_string_buffer(256)
    rc = L.gbsdf_selftest(1, 0, C.byref(res), err, len(err))
    assert rc == 0, err.value
    assert res.value == 0, f"{res.value} tile elements misplaced"
