"""CPU checks of librfk: it loads, exports every symbol of include/*.h, and
its host logic (database, DSL translation, genome layout, codegen, NVRTC
compile for sm_103a) works without a device."""
import ctypes
import json
import re
import zlib
import base64
from pathlib import Path

import numpy as np
import pytest

from oracle.build_ref import REFERENCE_ROOT as REFERENCE
from refraktor_gb300 import librefrakt as lr
from refraktor_gb300 import synthetic as syn
from refraktor_gb300 import _lib
from oracle import oracle as orc

ROOT = Path(__file__).resolve().parent.parent


def header_symbols():
    decl = re.compile(r"^(?:const\s+)?[a-z_0-9]+\s*\*?\s*(rfk_[a-z0-9_]+)\s*\(", re.M)
    syms = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        syms |= set(decl.findall(h.read_text()))
    return sorted(syms)


def test_exports_every_declared_symbol():
    L = ctypes.CDLL(str(_lib._LIB_PATH))
    syms = header_symbols()
    assert len(syms) > 30
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    # and the Python mirror binds all of them
    assert set(syms) <= set(_lib.SIGNATURES), set(syms) - set(_lib.SIGNATURES)


def test_version_and_error_channel():
    L = _lib.lib()
    assert L.rfk_version() >= 100
    h = ctypes.c_void_p()
    assert L.rfk_db_load(b"/nonexistent", ctypes.byref(h)) == 2
    assert b"cannot open" in L.rfk_last_error()


def test_bundled_db(db):
    names = db.variations()
    for n in syn.HD_SET + ["fisheye", "bubble", "gaussian_blur", "julian", "waves"]:
        assert n in names
    assert db.hash() != 0


def test_reference_db_loads_and_translates(ref_config):
    rdb = lr.flamedb(ref_config)
    names = rdb.variations()
    assert len(names) == 99
    for n in names:
        src = rdb.variation_source(n)
        assert "do {" in src


def _all_variations_flame(db, names, per_xform=6):
    xfs = []
    for i in range(0, len(names), per_xform):
        chunk = names[i:i + per_xform]
        vars_ = {}
        for n in chunk:
            d = lr.flame  # noqa
            vars_[n] = 0.1
        xfs.append({"weight": 1.0, "color": 0.5, "color_speed": 0.5, "opacity": 1.0,
                    "vchain": [{"transform": [1, 0, 0, 1, 0.1, -0.1], "mod_x": 0, "mod_y": 0, "mod_scale": 1,
                                "mod_rotate": 0, "variations": vars_}]})
    g = syn.plain_flame(0)
    g["xforms"] = xfs
    return g


def _with_params(db_obj, g):
    """Fill every variation that has ordinary parameters with its parameter object."""
    for xf in g["xforms"]:
        for vl in xf["vchain"]:
            for n in list(vl["variations"]):
                src = db_obj.variation_source(n)
                params = sorted(set(re.findall(r"\bP_([A-Za-z0-9_]+)\b", src)))
                if params:
                    vl["variations"][n] = {"weight": 0.1, "parameters": {}}
    return g


def test_nvrtc_compiles_every_bundled_variation(db):
    names = db.variations()
    g = _all_variations_flame(db, names)
    # variations with parameters need a parameter object; defaults fill the rest
    f = lr.flame.from_json(db, _with_params(db, g))
    log = lr.compile_check(db, f, "sm_103a")
    assert "error" not in log.lower()
    log = lr.compile_check(db, f, "sm_103a", precise_math=1)
    assert "error" not in log.lower()


def test_nvrtc_compiles_every_reference_variation(ref_config):
    rdb = lr.flamedb(ref_config)
    g = _all_variations_flame(rdb, rdb.variations(), per_xform=10)
    f = lr.flame.from_json(rdb, _with_params(rdb, g))
    lr.compile_check(rdb, f, "sm_103a")


def test_pack_sample_matches_oracle(db):
    for g in [syn.plain_flame(0), syn.plain_flame(3), syn.hd_flame(0), syn.hd_flame(5)]:
        g = dict(g, rotate=37.5, center_x=0.3, center_y=-0.2, mod_hue=20.0, mod_sat=-0.1)
        g["xforms"][0]["vchain"][0]["mod_rotate"] = 15.0
        g["xforms"][0]["vchain"][0]["mod_scale"] = 0.8
        f = lr.flame.from_json(db, g)
        for (w, h) in [(512, 512), (1920, 1080), (7, 3)]:
            a = f.pack_sample(w, h)
            b = orc.pack_sample(g, w, h)
            np.testing.assert_allclose(a, b, rtol=0, atol=1e-12)
        assert f.size_reals() == orc.size_reals(g)
        assert f.affine_indices() == orc.affine_indices(g)


def test_precalc_slots_and_params_layout(db):
    g = syn.plain_flame(0)
    g["xforms"][0]["vchain"][0]["variations"] = {
        "julian": {"weight": 0.5, "parameters": {"power": 3.0, "dist": 0.7}}, "linear": 0.25}
    f = lr.flame.from_json(db, g)
    s = f.pack_sample(64, 64)
    base = 13 + 4
    # affine, then julian: weight, dist, power (sorted), 2 precalc zeros, then linear
    assert list(s[base + 6: base + 6 + 6]) == [0.5, 0.7, 3.0, 0.0, 0.0, 0.25]


def test_json_round_trip(db):
    g = syn.hd_flame(2)
    f = lr.flame.from_json(db, g)
    g2 = f.serialize()
    f2 = lr.flame.from_json(db, g2)
    np.testing.assert_array_equal(f.pack_sample(100, 80), f2.pack_sample(100, 80))
    assert f.structure_hash() == f2.structure_hash()


def test_zlib_palette_blob(db):
    g = syn.plain_flame(1)
    raw = np.array(g["palette"], dtype=np.float64).tobytes()
    g2 = dict(g, palette=base64.b64encode(zlib.compress(raw, 9)).decode())
    g3 = dict(g, palette=base64.b64encode(zlib.compress(raw, 0)).decode())
    a = lr.flame.from_json(db, g).pack_sample(32, 32)
    np.testing.assert_array_equal(a, lr.flame.from_json(db, g2).pack_sample(32, 32))
    np.testing.assert_array_equal(a, lr.flame.from_json(db, g3).pack_sample(32, 32))


@pytest.mark.parametrize("bad", [
    {"xforms": "nope"},
    {"palette": [[0, 0]]},
])
def test_bad_genomes_rejected(db, bad):
    g = dict(syn.plain_flame(0), **bad)
    with pytest.raises(_lib.RfkError) as e:
        lr.flame.from_json(db, g)
    assert e.value.code == 2


def test_unknown_variation_rejected(db):
    g = syn.plain_flame(0)
    g["xforms"][0]["vchain"][0]["variations"] = {"no_such_variation": 1.0}
    with pytest.raises(_lib.RfkError):
        lr.flame.from_json(db, g)


def test_structure_hash_ignores_values(db):
    a = syn.plain_flame(0)
    b = json.loads(json.dumps(a))
    b["xforms"][0]["weight"] = 0.9
    b["xforms"][1]["vchain"][0]["transform"][0] = 0.1
    assert lr.flame.from_json(db, a).structure_hash() == lr.flame.from_json(db, b).structure_hash()
    c = json.loads(json.dumps(a))
    c["xforms"][0]["vchain"][0]["variations"]["swirl"] = 0.2
    assert lr.flame.from_json(db, a).structure_hash() != lr.flame.from_json(db, c).structure_hash()


def test_fix_rotation_matches_oracle(db):
    rng = np.random.default_rng(0)
    g = syn.hd_flame(1)
    f = lr.flame.from_json(db, g)
    R = f.size_reals()
    ss = R + 768
    samples = np.concatenate([f.pack_sample(300, 200) for _ in range(5)])
    samples += rng.normal(0, 0.3, samples.shape)
    samples[R::3] = rng.uniform(0, 360, samples[R::3].shape)  # hues of the first sample
    aff = f.affine_indices()
    a = lr.fix_rotation(samples, ss, R, aff)
    b = orc.fix_rotation(samples, ss, R, aff)
    np.testing.assert_array_equal(a, b)


def test_flam3_import(db):
    xml = """<flames><flame name="t" size="640 480" center="0.1 -0.2" scale="120" rotate="10" brightness="3"
      gamma="2.5" vibrancy="0.8" highlight_power="1">
      <xform weight="0.7" color="0.2" spherical="0.5" julia="0.5" coefs="0.5 0.1 -0.1 0.5 0.2 0.3" post="1 0 0 1 0.5 0"/>
      <xform weight="0.3" color="0.9" linear="1" pre_blur="0.2" coefs="0.3 0 0 0.3 0 0"/>
      <finalxform color="0" color_speed="0" linear="1" coefs="1 0 0 1 0 0"/>
      <palette count="256" format="RGB">""" + "FF0000" * 128 + "00FF00" * 128 + """</palette>
      </flame></flames>"""
    f = lr.flame.import_flam3(db, xml)
    js = f.serialize()
    assert len(js["xforms"]) == 2 and "final_xform" in js
    assert len(js["xforms"][0]["vchain"]) == 2  # main + post
    assert len(js["xforms"][1]["vchain"]) == 2  # pre + main
    assert js["xforms"][1]["vchain"][0]["variations"] == {"gaussian_blur": 0.2}
    assert js["scale"] == pytest.approx(120 / 480)
    assert js["palette"][0] == pytest.approx([0.0, 1.0, 1.0])
    assert js["palette"][200] == pytest.approx([120.0, 1.0, 1.0])


def test_flam3_reference_fixture(db):
    p = REFERENCE / "assets/flames_test/electricsheep.247.50049.flam3"
    if not p.exists():
        pytest.skip("reference fixture not present")
    f = lr.flame.import_flam3(db, p.read_text())
    js = f.serialize()
    assert len(js["xforms"]) == 4
    assert sorted(js["xforms"][1]["vchain"][0]["variations"]) == ["disc", "fisheye", "heart", "spherical"]
    assert len(js["xforms"][1]["vchain"]) == 2  # post affine -> linear vlink
    assert js["gamma"] == 4 and js["brightness"] == pytest.approx(64.0783)
    lr.compile_check(db, f, "sm_103a")


def test_db_add_remove_and_queries():
    """flamedb::add_or_update_variation / add_or_update_common / remove_* /
    is_* (flame_info.h:69-129) on a private database."""
    fdb = lr.flamedb()
    h0 = fdb.hash()
    assert fdb.is_variation("julian") and fdb.is_parameter("julian", "power") and fdb.is_parameter("julian", "rN")
    assert not fdb.is_parameter("julian", "nope") and not fdb.is_variation("scaled_linear")
    assert fdb.is_common("phi") and not fdb.is_common("double_r")
    fdb.add_or_update_common("double_r", "2.0 * common.sqrt")
    fdb.add_or_update_variations(
        "scaled_linear:\n"
        "  param:\n"
        "    s: {default: 2.0}\n"
        "  src: |-\n"
        "    result += weight * param.s * p;\n"
        "ring_r: result += weight * common.double_r * p;\n")
    assert fdb.is_common("double_r") and fdb.is_variation("scaled_linear") and fdb.is_variation("ring_r")
    assert fdb.is_parameter("scaled_linear", "s")
    h1 = fdb.hash()
    assert h1 != h0
    # a genome can use the new variation, and its generated code reads its parameter
    g = syn.plain_flame(0)
    g["xforms"][0]["vchain"][0]["variations"] = {"scaled_linear": {"weight": 0.5, "s": 3.0}}
    f = lr.flame.from_json(fdb, g)
    assert f.size_reals() > 0
    # invalid bodies are rejected and leave the database as it was
    with pytest.raises(_lib.RfkError) as e:
        fdb.add_or_update_variations("broken: result += weight * param.missing * p;\n")
    assert e.value.code == 2 and not fdb.is_variation("broken") and fdb.hash() == h1
    with pytest.raises(_lib.RfkError):
        fdb.add_or_update_common("bad", "p.x +")
    assert fdb.remove_variation("ring_r") and not fdb.remove_variation("ring_r")
    assert not fdb.is_variation("ring_r") and fdb.hash() != h1
    assert fdb.remove_common("double_r") and not fdb.is_common("double_r")
    assert fdb.remove_variation("scaled_linear")
    assert fdb.hash() == h0  # back to the loaded definitions


def test_denoiser_weight_file_reader(tmp_path):
    """rfk_denoiser_read_params reads the committed weights and other .npz
    layouts (stored or compressed, float16 or float32) exactly as numpy."""
    from refraktor_gb300 import denoise as dn

    path = Path(lr.__file__).resolve().parent / "workloads" / "denoiser_weights.npz"
    np.testing.assert_array_equal(dn.read_params(path), np.load(path)["params"].astype(np.float32))
    halves = np.array([0.0, -0.0, 1.0, -2.5, 6.1e-5, 5.96e-8, -3.0e-7, 65504.0, np.inf, -np.inf], dtype=np.float16)
    np.savez(tmp_path / "stored.npz", params=halves)
    np.testing.assert_array_equal(dn.read_params(tmp_path / "stored.npz"), halves.astype(np.float32))
    full = np.random.default_rng(0).standard_normal(5000).astype(np.float32)
    np.savez_compressed(tmp_path / "deflated.npz", params=full)
    np.testing.assert_array_equal(dn.read_params(tmp_path / "deflated.npz"), full)
    np.savez(tmp_path / "other.npz", weights=full)
    with pytest.raises(_lib.RfkError):
        dn.read_params(tmp_path / "other.npz")  # no params member
    with pytest.raises(_lib.RfkError):
        dn.read_params(tmp_path / "missing.npz")


def test_denoiser_factory_names():
    """denoiser::make by name (factory.h:71-98): the registry lists the U-Net,
    and an unknown name fails before any device work."""
    from refraktor_gb300 import denoise as dn

    assert dn.names() == ["rfkt::gb300_unet_denoiser"]
    with pytest.raises(_lib.RfkError) as e:
        dn.denoiser.make("rfkt::oidn_denoiser")
    assert e.value.code == 1 and "unknown denoiser" in str(e.value)
