"""Host logic of the brick-shape autotuner (no GPU)."""
import torch

from framework_gb300 import autotune


def test_signature_groups_by_size_and_dtype():
    a = [dict(volume=torch.zeros((17, 33, 65))), dict(volume=torch.zeros((9, 9, 9), dtype=torch.int16))]
    b = [dict(volume=torch.zeros((17, 33, 66))), dict(volume=torch.zeros((9, 9, 10), dtype=torch.int16))]
    c = [dict(volume=torch.zeros((170, 33, 65))), dict(volume=torch.zeros((9, 9, 9), dtype=torch.int16))]
    assert autotune.batch_signature(a) == autotune.batch_signature(b)
    assert autotune.batch_signature(a) != autotune.batch_signature(c)
    assert "float32+int16" in autotune.batch_signature(a)
    assert autotune.batch_signature([dict(volume=torch.zeros((1, 5, 5)))]).endswith("h=-1:1")


def test_cache_roundtrip(tmp_path):
    p = str(tmp_path / "sub" / "t.json")
    assert autotune._load(p) == {}
    autotune._save(p, {"k": {"planes": 8}})
    assert autotune._load(p) == {"k": {"planes": 8}}


def test_stream_handle_mapping():
    import framework_gb300 as fg
    # torch's legacy default stream (0) must not become the library's own stream (NULL)
    assert fg._stream_handle(0) == 0x1
    assert fg._stream_handle(0x7f00) == 0x7f00

    class S:
        cuda_stream = 0
    assert fg._stream_handle(S()) == 0x1
