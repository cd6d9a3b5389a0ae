"""Structure alignment (rfk_flames_align): genomes of different structure get
one structure and still map every point exactly as before. Checked on the CPU
with the FP64 oracle's single-map application of the packed genomes."""
import copy

import numpy as np
import pytest

from oracle import oracle as orc
from refraktor_gb300 import librefrakt as lr
from refraktor_gb300 import synthetic as syn


def _genomes():
    gs = [syn.hd_flame(11, n_xforms=3, final=False), syn.hd_flame(12, n_xforms=6, final=True),
          syn.hd_flame(13, n_xforms=12, final=False, var_set=["linear", "spherical", "swirl", "julia"])]
    # a two-vlink xform: the others must be padded at that position
    extra = copy.deepcopy(gs[0]["xforms"][1]["vchain"][0])
    extra["variations"] = {"sinusoidal": 0.7}
    gs[0]["xforms"][1]["vchain"].append(extra)
    # a vlink with a half-turn pad variation next to it
    gs[1]["xforms"][0]["vchain"].append({"transform": [0.9, 0.1, -0.2, 0.8, 0.05, -0.1], "mod_x": 0, "mod_y": 0,
                                         "mod_scale": 1, "mod_rotate": 0, "variations": {"linear": 0.5, "polar": 0.5}})
    return gs


def _points(n=257, seed=0):
    rng = np.random.default_rng(seed)
    p = rng.uniform(-1.5, 1.5, size=(n, 3))
    p[:, 2] = rng.uniform(0, 1, n)
    return p


@pytest.mark.parametrize("by_weight", [False, True])
def test_aligned_genomes_share_one_structure(db, by_weight):
    gs = _genomes()
    fs = [lr.flame.from_json(db, g) for g in gs]
    assert len({f.structure_hash() for f in fs}) == 3
    al = lr.align_flames(db, fs, by_weight=by_weight)
    assert len({f.structure_hash() for f in al}) == 1
    assert len({f.size_reals() for f in al}) == 1
    nx = len(al[0].serialize()["xforms"])
    assert nx == (21 if by_weight else 12)
    for f in al:
        assert f.serialize().get("final_xform") is not None


@pytest.mark.parametrize("by_weight", [False, True])
def test_aligned_genomes_map_points_exactly_as_before(db, by_weight):
    """Every original xform (and final xform) of every genome maps points
    bit-identically after alignment: added variations weigh 0 and are skipped,
    padding vlinks are exact identities (linear 1, or linear -1 after a -1
    affine). The xforms that do not belong to a genome weigh 0, so its xform
    pick distribution is unchanged, and a missing final xform becomes the
    identity."""
    gs = _genomes()
    fs = [lr.flame.from_json(db, g) for g in gs]
    al = lr.align_flames(db, fs, by_weight=by_weight)
    pts = _points()
    first = 0
    for g, a in zip(gs, al):
        ga = a.serialize()
        p0 = orc.pack_sample(g, 64, 48)
        pa = orc.pack_sample(ga, 64, 48)
        # the library's packing of the aligned genome is the oracle's
        np.testing.assert_array_equal(a.pack_sample(64, 48)[: a.size_reals()], pa[: a.size_reals()])
        nx = len(g["xforms"])
        off = first if by_weight else 0
        for k in range(nx):
            np.testing.assert_array_equal(orc.apply_many(ga, pa, off + k, pts), orc.apply_many(g, p0, k, pts))
        wts = [x["weight"] for x in ga["xforms"]]
        mine = set(range(off, off + nx))
        assert all(wts[i] == 0.0 for i in range(len(wts)) if i not in mine)
        assert [wts[i] for i in sorted(mine)] == [x["weight"] for x in g["xforms"]]
        nxa = len(ga["xforms"])
        fin_a = orc.apply_many(ga, pa, nxa, pts)
        if g.get("final_xform") is not None:
            np.testing.assert_array_equal(fin_a, orc.apply_many(g, p0, nx, pts))
        else:
            np.testing.assert_array_equal(fin_a[:, :3], pts)
        if by_weight:
            first += nx


def test_padder_follows_pad_tags(db):
    """make_padder picks the identity form from the padded vlink's variations:
    linear 1 by default, linear -1 after a -1 affine for a half-turn variation
    (polar), and the rest of the variations at weight 0."""
    g = syn.hd_flame(3, n_xforms=2, final=False, var_set=["linear", "sinusoidal", "spherical"])
    h = copy.deepcopy(g)
    h["xforms"][0]["vchain"].append({"transform": [1, 0, 0, 1, 0, 0], "mod_x": 0, "mod_y": 0, "mod_scale": 1,
                                     "mod_rotate": 0, "variations": {"polar": 0.6, "swirl": 0.4}})
    al = lr.align_flames(db, [lr.flame.from_json(db, g), lr.flame.from_json(db, h)])
    pad = al[0].serialize()["xforms"][0]["vchain"][1]
    assert pad["transform"][:4] == [-1.0, 0.0, 0.0, -1.0]
    v = pad["variations"]
    w = {n: (x["weight"] if isinstance(x, dict) else x) for n, x in v.items()}
    assert w == {"linear": -1.0, "polar": 0.0, "swirl": 0.0}


def test_align_rejects_nothing_and_keeps_single_genome(db):
    f = lr.flame.from_json(db, syn.plain_flame(2))
    (a,) = lr.align_flames(db, [f])
    assert a.structure_hash() == f.structure_hash()
    np.testing.assert_array_equal(a.pack_sample(32, 32), f.pack_sample(32, 32))
