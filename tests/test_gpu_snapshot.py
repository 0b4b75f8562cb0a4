"""Background snapshot writer: the files hold exactly the reference's datasets of the state
at submission (save_data.py:7-32), although the batch keeps stepping while they are
copied out and written."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_writer_snapshots_the_state_at_submission(cuda, tmp_path):
    from pmgpu import ics
    from pmgpu.batch import Batch
    from pmgpu.config import Config
    from pmgpu.snapshot import SnapshotWriter, host_snapshot, read_file
    cfg = Config(n_parts=64, n_cells=128, box_size=200.0, random_seed=9, steps=100)
    b = Batch()
    sid = b.add(cfg, *ics.initial_conditions(cfg))
    w = SnapshotWriter(cfg.box_size, cfg.n_cells, cfg.h0, directory=str(tmp_path))
    expect = {}
    for k in range(3):
        b.step(7)
        pos_h, vel_h, a, _ = b.get(sid)
        pos_d, vel_d, a2, _ = b.get(sid, device=True)
        assert a2 == a
        w.submit(k, pos_d, vel_d, a)
        expect[k] = host_snapshot(pos_h, vel_h, a, cfg.box_size, cfg.n_cells, cfg.h0)
    b.step(20)  # keeps running while the writes complete
    paths = w.close()
    b.close()
    assert len(paths) == 3
    for k, path in enumerate(paths):
        got = read_file(path)
        for name, arr in expect[k].items():
            assert np.array_equal(got[name], arr), (k, name)
