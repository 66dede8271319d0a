"""bench.py under a multi-process launch, on CPU (world size 2, no GPU touched): the GPU arm
refuses to run with more than one rank, because its tensor-core kernel is for single-GPU
processes only; the reference arm prints only on rank 0."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _launch(rank, world, *extra):
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
               MASTER_ADDR="127.0.0.1", MASTER_PORT="29531")
    return subprocess.Popen([sys.executable, os.path.join(ROOT, "bench.py"), *extra],
                            cwd=ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                            text=True)


def test_two_ranks_are_refused():
    procs = [_launch(r, 2, "--gpus", "2") for r in range(2)]
    outs = [p.communicate(timeout=120) for p in procs]
    assert [p.returncode for p in procs] == [2, 2]
    assert all(o[0] == "" for o in outs)  # no benchmark line
    assert "one GPU only" in outs[0][1]
    assert outs[1][1] == ""


def test_gpus_flag_above_one_is_refused():
    p = _launch(0, 1, "--gpus", "4")
    out, err = p.communicate(timeout=120)
    assert p.returncode == 2 and out == "" and "one GPU only" in err


def test_reference_arm_silent_off_rank_zero(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        steps, warmup, cpu_rows = 1, 0, 1
    assert bench.run_reference(Args(), rank=1, world=2) is None
    assert capsys.readouterr().out == ""
