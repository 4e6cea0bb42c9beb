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
