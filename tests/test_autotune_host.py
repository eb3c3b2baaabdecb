"""Host logic of the launch-shape tuner (no GPU): the JSON cache of picks."""
import json


def test_cache_round_trip_with_a_bare_file_name(tmp_path, monkeypatch):
    """MPF3D_TUNING_CACHE may name a file in the working directory."""
    from mpf3d import autotune
    monkeypatch.chdir(tmp_path)
    monkeypatch.setenv("MPF3D_TUNING_CACHE", "tune.json")
    db = {"GB300|256x256x256": {"config": [8, 8, 4, 256, 32, 64], "sweep_tma": True}}
    autotune._store(db)
    assert json.loads((tmp_path / "tune.json").read_text()) == db
    assert autotune._load() == db


def test_cache_in_a_new_directory_and_a_broken_file(tmp_path, monkeypatch):
    from mpf3d import autotune
    path = tmp_path / "a" / "b" / "tuning.json"
    monkeypatch.setenv("MPF3D_TUNING_CACHE", str(path))
    assert autotune._load() == {}
    autotune._store({"k": {"config": [4, 8, 8, 256, 8, 128]}})
    assert autotune._load() == {"k": {"config": [4, 8, 8, 256, 8, 128]}}
    path.write_text("{not json")
    assert autotune._load() == {}


def test_make_orders_the_six_fields():
    from mpf3d import autotune
    t = autotune.make([2, 16, 3, 128, 5, 64])
    assert (t.sweep_zb, t.sweep_by, t.general_blocks_per_sm, t.general_threads, t.iface_blocks_per_sm,
            t.iface_threads) == (2, 16, 3, 128, 5, 64)
