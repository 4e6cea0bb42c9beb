"""Binary model cache (smx_save_model_cache): host-only, no GPU.

JSON -> cache -> cache must be byte-identical (every packed table and scalar
survives the round trip), a corrupt or truncated cache is rejected, and loading the
cache is much faster than parsing the JSON.
"""
import os
import time

import pytest

from symmetrix_gb300 import _lib, save_model_cache


@pytest.mark.parametrize("variant", ["plain", "density_zbl"])
def test_cache_round_trip_is_exact(engine_lib, small_model_path, tmp_path, variant):
    from symmetrix_gb300.synth.model import CONFIGS, make_model, write_model
    src = small_model_path
    if variant == "density_zbl":
        src = write_model(make_model(**dict(CONFIGS["small"], num_knots=40), seed=2, density_scaled=True, zbl=True),
                          str(tmp_path / "dz.json"))
    a, b = str(tmp_path / "a.smxb"), str(tmp_path / "b.smxb")
    t = time.time()
    save_model_cache(src, a)
    t_json = time.time() - t
    t = time.time()
    save_model_cache(a, b)
    t_cache = time.time() - t
    print(f"from JSON {t_json:.3f} s, from cache {t_cache:.3f} s, {os.path.getsize(a) / 1e6:.1f} MB")
    assert open(a, "rb").read() == open(b, "rb").read()


def test_corrupt_cache_is_rejected(engine_lib, small_model_path, tmp_path):
    a, bad = str(tmp_path / "a.smxb"), str(tmp_path / "bad.smxb")
    save_model_cache(small_model_path, a)
    data = open(a, "rb").read()
    open(bad, "wb").write(data[: len(data) // 2])
    with pytest.raises(RuntimeError):
        save_model_cache(bad, str(tmp_path / "c.smxb"))
    with pytest.raises(RuntimeError):
        save_model_cache(str(tmp_path / "missing.json"), str(tmp_path / "d.smxb"))


MALFORMED = {
    "missing key": (lambda m: m.pop("r_cut"), "missing key 'r_cut'"),
    "r_cut zero": (lambda m: m.update(r_cut=0.0), "r_cut must be positive"),
    "spline step negative": (lambda m: m.update(radial_spline_h=-0.1), "radial_spline_h"),
    "knots short of r_cut": (lambda m: m.update(radial_spline_h=m["radial_spline_h"] * 0.5), "radial_spline_h"),
    "ragged spline row": (lambda m: m["radial_spline_values_1"][0].pop(), "ragged array"),
    "l_max": (lambda m: m.update(l_max=4), "l_max must be 3"),
    "channels": (lambda m: m.update(num_channels=48), "num_channels"),
    "species tables": (lambda m: m["atomic_energies"].pop(), "species table sizes"),
    "H1_weights size": (lambda m: m["H1_weights"].pop(), "H1_weights size"),
    "monomial variable": (lambda m: m["M0_monomials"]["0"][3].__setitem__(0, 99), "monomial variable out of range"),
    "coupling index": (lambda m: m["Phi1_lme"].__setitem__(0, 999), "coupling index out of range"),
    "readout size": (lambda m: m["readout_1_weights"].pop(), "readout_1_weights size"),
}


@pytest.mark.parametrize("case", sorted(MALFORMED))
def test_malformed_model_is_rejected(engine_lib, small_model_path, tmp_path, case):
    """The loader checks what the reference's load_from_json (mace.cpp:905-1030) trusts:
    every malformation raises with a message naming it, before anything reaches a GPU."""
    import json
    mutate, message = MALFORMED[case]
    m = json.load(open(small_model_path))
    mutate(m)
    bad = str(tmp_path / "bad.json")
    json.dump(m, open(bad, "w"))
    with pytest.raises(RuntimeError, match=message):
        save_model_cache(bad, str(tmp_path / "bad.smxb"))


def test_truncated_json_is_rejected(engine_lib, small_model_path, tmp_path):
    bad = str(tmp_path / "cut.json")
    open(bad, "w").write(open(small_model_path).read()[:1000])
    with pytest.raises(RuntimeError, match="not valid JSON"):
        save_model_cache(bad, str(tmp_path / "cut.smxb"))


def test_cli_generates_and_caches_a_model(engine_lib, tmp_path):
    """`python -m symmetrix_gb300.cli gen-model` / `cache` (the commands the profile
    summaries use) on the CPU: the cache of the generated JSON equals the cache of
    the cache."""
    from symmetrix_gb300.cli import main
    js, a, b = str(tmp_path / "m.json"), str(tmp_path / "a.smxb"), str(tmp_path / "b.smxb")
    main(["gen-model", js, "--config", "small", "--knots", "20", "--zbl"])
    main(["cache", js, a])
    main(["cache", a, b])
    assert open(a, "rb").read() == open(b, "rb").read()
