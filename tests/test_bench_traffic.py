"""bench.profile_traffic: the DRAM bytes per launch that the bench reports as
roofline.traffic come from a committed ncu capture keyed to the sha256 of
the kernel sources it was made on, and are withheld once those sources
change.  Checked on the CPU against a temporary copy of the tree."""
import json
import os
import shutil
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench_copy(tmp_path):
    """bench.py plus the kernel sources it hashes, in a scratch tree."""
    sys.path.insert(0, ROOT)
    import bench
    dst = tmp_path / "tree"
    (dst / "framework_gb300" / "csrc").mkdir(parents=True)
    (dst / "profiles").mkdir()
    for name in bench.TRAFFIC_SOURCES:
        shutil.copy(os.path.join(ROOT, "framework_gb300", "csrc", name), dst / "framework_gb300" / "csrc" / name)
    return bench, dst


def test_traffic_reported_while_sources_match(tmp_path, monkeypatch):
    bench, dst = _bench_copy(tmp_path)
    monkeypatch.setattr(bench, "ROOT", str(dst))
    rec = {"sources_sha256": bench.kernel_sources_sha256(), "noise1024:emit": 123, "batch256:count": 45}
    (dst / "profiles" / "traffic.json").write_text(json.dumps(rec))
    assert bench.profile_traffic("noise1024") == 123
    assert bench.profile_traffic("batch256", kernel="count") == 45
    assert bench.profile_traffic("served64") is None        # never captured


def test_traffic_withheld_after_a_source_change(tmp_path, monkeypatch, capsys):
    bench, dst = _bench_copy(tmp_path)
    monkeypatch.setattr(bench, "ROOT", str(dst))
    rec = {"sources_sha256": bench.kernel_sources_sha256(), "noise1024:emit": 123}
    (dst / "profiles" / "traffic.json").write_text(json.dumps(rec))
    src = dst / "framework_gb300" / "csrc" / bench.TRAFFIC_SOURCES[0]
    src.write_text(src.read_text() + "\n// changed\n")
    assert bench.profile_traffic("noise1024") is None
    assert "other kernel sources" in capsys.readouterr().err


def test_traffic_absent_record(tmp_path, monkeypatch):
    bench, dst = _bench_copy(tmp_path)
    monkeypatch.setattr(bench, "ROOT", str(dst))
    assert bench.profile_traffic("noise1024") is None


def test_committed_record_names_the_captured_workloads():
    """The committed record holds both sweeps of the default and the batched workloads."""
    d = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
    for key in ("noise1024:emit", "noise1024:count", "batch256:emit", "batch256:count"):
        assert isinstance(d[key], int) and d[key] > 0
    assert len(d["sources_sha256"]) == 64
