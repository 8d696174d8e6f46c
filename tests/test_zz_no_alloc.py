"""rp_contacts_noalloc (static device scratch, no allocation in the call) against rp_contacts on every
broad-phase pair of a settled pile pressed 3 mm into its supports, two calls in a row each: identical contacts in both builds. Kept
in its own file, collected last, so it runs after every other GPU test as well as alone."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_noalloc_contacts_match_rp_contacts(ext_built, precision):
    from rawphys import scenes as S
    sc = S.random_pile_scene(14, seed=21)
    w = ext_built.World(0, precision)
    w.load(sc)
    w.step(40)
    st = w.get_state()
    st[~sc.fixed, 1] -= 0.003          # resting bodies pushed 3 mm into their supports: contacts exist
    w.set_state(st)
    pairs = w.broad_pairs()
    assert len(pairs) > 0
    seen = 0
    for a, b in pairs:
        ref = w.contacts(int(a), int(b))
        for _ in range(2):
            got = w.contacts_noalloc(int(a), int(b))
            assert np.array_equal(got, ref), (precision, a, b)
        seen += len(ref) > 0
    assert seen > 0, "no pair in contact"
    w.close()


def test_noalloc_rejects_cap_beyond_scratch_and_unbuilt_world(ext_built):
    from rawphys import scenes as S
    sc = S.random_pile_scene(4, seed=2)
    w = ext_built.World(0, "fp32")
    w.load(sc)
    with pytest.raises(ext_built.RPError, match="not built"):
        w.contacts_noalloc(0, 1)
    w.step(1)
    with pytest.raises(ext_built.RPError, match="static scratch"):
        w.contacts_noalloc(0, 1, cap=65)
    w.close()


def test_noalloc_partial_cap_writes_only_cap_rows(ext_built):
    """A pair with more contacts than cap: the count is the full total, only the first cap rows are
    written (cap 1: the first contact; cap 0: nothing), through the raw C-ABI call."""
    import ctypes as C
    from rawphys import scenes as S
    sc = S.random_pile_scene(14, seed=21)
    w = ext_built.World(0, "fp32")
    w.load(sc)
    w.step(40)
    st = w.get_state()
    st[~sc.fixed, 1] -= 0.003
    w.set_state(st)
    multi = None
    for a, b in w.broad_pairs():
        ref = w.contacts(int(a), int(b))
        if len(ref) >= 2:
            multi = (int(a), int(b), ref)
            break
    assert multi is not None, "no pair with two or more contacts"
    a, b, ref = multi
    for cap in (1, 0):
        out = np.full(9 * 4, 12345.0)
        n = C.c_uint32(0)
        rc = w.lib.rp_contacts_noalloc(w.h, a, b, out.ctypes.data_as(C.POINTER(C.c_double)), cap, C.byref(n))
        assert rc == 0
        assert n.value == len(ref)
        assert np.array_equal(out[:9 * cap].reshape(-1, 9), ref[:cap])
        assert np.all(out[9 * cap:] == 12345.0), "rows beyond cap were written"
    w.close()


def test_noalloc_uploads_host_edits_without_a_step(ext_built):
    """A velocity edit after the last step is uploaded by the call itself (no allocation): the
    query then answers on the world's current state instead of refusing."""
    from rawphys import scenes as S
    sc = S.random_pile_scene(6, seed=3)
    w = ext_built.World(0, "fp32")
    w.load(sc)
    w.step(2)
    a, b = (int(x) for x in w.broad_pairs()[0])
    w.set_velocity(int(np.nonzero(~sc.fixed)[0][0]), [0.0, 1.0, 0.0], [0.0, 0.0, 0.0])
    got = w.contacts_noalloc(a, b)
    assert np.array_equal(got, w.contacts(a, b))
    w.close()
