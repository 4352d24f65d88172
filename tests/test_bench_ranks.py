"""bench.py under more than one rank: one image, one GPU.

The GPU arm does no work on any rank when WORLD_SIZE > 1 (or --gpus > 1):
rank 0 prints one JSON line that says why, other ranks print nothing, and all
exit 0 without loading the library.  The reference arm (host cores only) runs
on rank 0 alone; other ranks exit 0 without work.  Both arms' ``config``
dicts are the same function of the workload.
"""
import argparse
import io
import json
import sys
from contextlib import redirect_stdout

import pytest


def _main(monkeypatch, argv, rank, world):
    import bench
    monkeypatch.setenv("RANK", str(rank))
    monkeypatch.setenv("WORLD_SIZE", str(world))
    monkeypatch.setenv("LOCAL_RANK", str(rank))
    monkeypatch.setattr(sys, "argv", ["bench.py"] + argv)
    buf = io.StringIO()
    with redirect_stdout(buf):
        rc = bench.main()
    return rc, buf.getvalue()


@pytest.mark.parametrize("rank", [0, 1])
def test_gpu_arm_refuses_more_than_one_rank(monkeypatch, rank):
    rc, out = _main(monkeypatch, ["--gpus", "2", "--steps", "2", "--warmup", "1"], rank, 2)
    assert rc == 0
    if rank == 0:
        line = json.loads(out.strip())
        assert line["n_gpus"] == 2 and line["value"] is None
        assert "one GPU per call" in line["unavailable"]
    else:
        assert out == ""


def test_gpu_arm_refuses_gpus_flag_on_one_rank(monkeypatch):
    rc, out = _main(monkeypatch, ["--gpus", "4"], 0, 1)
    assert rc == 0 and json.loads(out)["unavailable"]


def test_reference_arm_other_ranks_idle():
    import bench
    args = argparse.Namespace(steps=2, warmup=1, impl="reference", gpus=2)
    assert bench.run_reference(args, 2, 1) == 0             # rank 1: no work, exit 0


def test_config_identical_in_both_arms():
    import bench
    from elphbolt_gb300 import synthetic as S
    wd = S.make_wannier(S.make_crystal_si_like(), 4, supercell=(2, 2, 2), seed=11)
    req = S.si_like_request(wd, (4, 4, 4))
    c = bench.config_dict(wd, req)
    assert c == bench.config_dict(wd, req)
    assert not {"window_k", "initial_states", "vertices_per_step"} & set(c)
