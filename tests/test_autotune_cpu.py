"""The autotuner's host side (candidates, table merge, device matching) and the
tile table's argument checks, without a GPU."""
import json

import pytest

from wannier_tools_gb300 import _lib, autotune


def test_candidates():
    assert autotune.candidates("fp64", 40) == [128, 256, 512]
    assert autotune.candidates("fp64", 119) == [128, 256, 512]
    assert autotune.candidates("fp64", 120) == []          # inverse in global memory: 256 threads
    assert autotune.candidates("mixed", 112) == [24, 32, 40]
    assert autotune.candidates("mixed", 264) == [24, 32, 40]   # 6 accumulators: at most 40 columns
    assert autotune.candidates("mixed", 16) == []
    assert autotune.candidates("mixed", 321) == []
    with pytest.raises(ValueError):
        autotune.candidates("tf32", 40)


def test_sample_grows_at_small_ndim():
    assert autotune.default_solves(152, 112) == 304
    assert autotune.default_solves(152, 264) == 304
    assert autotune.default_solves(152, 40) == round(304 * (112 / 40) ** 3)
    assert autotune.default_solves(152, 8) == 16384


def test_model_shape_per_ndim():
    assert autotune.shape_for(112) == (56, 2)
    assert autotune.shape_for(264) == (132, 2)
    assert autotune.shape_for(39) == (13, 3)
    assert autotune.shape_for(7) == (7, 1)


def test_device_key_drops_memory():
    info = "NVIDIA GB300, 152 SMs, cc 10.3, 275.0 GiB"
    assert autotune.device_key(info) == "NVIDIA GB300, 152 SMs, cc 10.3"


def test_table_merge_and_lookup(tmp_path):
    path = tmp_path / "tiles.json"
    dev = "NVIDIA GB300, 152 SMs, cc 10.3"
    autotune.save({"entries": {"fp64": {"40": 128}, "mixed": {"112": 40}},
                   "ms": {"fp64": {"40": {"128": 1.0, "256": 1.2}}, "mixed": {}}}, dev, path)
    autotune.save({"entries": {"mixed": {"264": 32}}, "ms": {"mixed": {"264": {"32": 9.0}}}}, dev, path)
    table = json.loads(path.read_text())
    got = autotune.entries_for(table, dev)
    assert got == {"fp64": {40: 128}, "mixed": {112: 40, 264: 32}}
    assert autotune.entries_for(table, "another device") == {}


def test_committed_table_is_valid():
    if not autotune.TABLE.exists():
        pytest.skip("no tile table committed")
    table = json.loads(autotune.TABLE.read_text())
    for dev in table["devices"]:
        for form, ent in autotune.entries_for(table, dev).items():
            for ndim, v in ent.items():
                assert v in autotune.candidates(form, ndim), (dev, form, ndim, v)


def test_tile_arguments_are_checked(built_lib):
    lib = built_lib
    assert lib.wtg_tile_set(0, 40, 100) == _lib.WTG_EINVAL           # not 128/256/512
    assert lib.wtg_tile_set(1, 112, 52) == _lib.WTG_EINVAL           # not a multiple of 8
    assert lib.wtg_tile_set(1, 264, 48) == _lib.WTG_EINVAL           # above 40 columns
    assert lib.wtg_tile_set(1, 400, 32) == _lib.WTG_EINVAL           # beyond the mixed kernel
    assert lib.wtg_tile_set(2, 40, 0) == _lib.WTG_EINVAL
    assert lib.wtg_tile_set(0, 0, 0) == _lib.WTG_EINVAL
    from wannier_tools_gb300 import api
    assert api.get_tile(1, 112) == (40, 40)
    api.set_tile(1, 112, 32)
    try:
        assert api.get_tile(1, 112) == (32, 40)
    finally:
        api.set_tile(1, 112, 0)
    assert api.get_tile(0, 40) == (128, 128)
    assert api.get_tile(0, 200) == (256, 256)


def test_engine_graph_calls_check_the_handle(built_lib):
    assert built_lib.wtg_engine_set_graphs(None, 1) == _lib.WTG_EINVAL
    assert built_lib.wtg_engine_graph_info(None, None, None) == _lib.WTG_EINVAL
