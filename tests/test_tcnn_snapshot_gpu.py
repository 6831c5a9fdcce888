"""tiny-cuda-nn Trainer snapshots (nmg_export_tcnn / nmg_import_tcnn) against
snapshots written by the reference's own serializer.

tests/golden/tcnn_golden.npz holds, for a small network (the reference preset
with a 2-level dense grid of base resolution 4: 13,408 parameters) and
parameters given by a fixed formula, the MessagePack bytes of the object
tcnn's Trainer::serialize builds (trainer.h:267-278), encoded by the
reference's vendored nlohmann::json::to_msgpack, once with "__half" and once
with "float" parameters. The library's exporter must write the same bytes
for the same parameters, and its importer must read those files back."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SNAPSHOT_CONFIG = dict(grid_levels=2, grid_base_resolution=4)


def table_values(n):
    i = np.arange(n, dtype=np.uint64)
    return (((i * np.uint64(2654435761)) % np.uint64(1 << 32)).astype(np.float64) / 2.0 ** 32 - 0.5).astype(np.float32)


@pytest.fixture(scope="module")
def tg():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "tcnn_golden.npz")))


def make_field(nmg):
    return nmg.GuidingField(nmg.config(nmg.PRESET_REFERENCE, path=nmg.PATH_FP32, **SNAPSHOT_CONFIG))


@pytest.mark.parametrize("ptype", ["__half", "float"])
def test_export_writes_the_reference_serializer_bytes(nmg, tg, tmp_path, ptype):
    import torch
    f = make_field(nmg)
    n = int(tg["snapshot_n_params"])
    assert f.n_params == n
    f.set_params(torch.from_numpy(table_values(n) * np.float32(0.2)).cuda())
    path = tmp_path / "net.msgpack"
    f.export_tcnn(path, ptype)
    want = tg["snapshot_half" if ptype == "__half" else "snapshot_float"].tobytes()
    assert path.read_bytes() == want
    f.close()


@pytest.mark.parametrize("ptype", ["__half", "float"])
def test_import_reads_the_reference_serializer_bytes(nmg, tg, tmp_path, ptype):
    f = make_field(nmg)
    path = tmp_path / "ref.msgpack"
    path.write_bytes(tg["snapshot_half" if ptype == "__half" else "snapshot_float"].tobytes())
    f.import_tcnn(path)
    want = table_values(f.n_params) * np.float32(0.2)
    if ptype == "__half":
        want = want.astype(np.float16).astype(np.float32)
    for which in (0, 1):  # both parameter copies are set
        assert np.array_equal(f.get_params(which).cpu().numpy(), want)
    f.check_errors()
    f.close()
