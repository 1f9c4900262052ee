"""The work queue of the dataflow kernels (lcg_host::queue_order,
engine_prep.hh) on CPU, through a small driver compiled from
tests/cpp/queue_order_demo.cu."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def queue_demo():
    from locarna_gb300.build import GENCODE, NVCC, OUT, _run
    exe = os.path.join(OUT, "queue_order_demo")
    _run([NVCC, GENCODE, "-std=c++17", "-O1", os.path.join(ROOT, "tests", "cpp", "queue_order_demo.cu"), "-o", exe])
    return exe


@pytest.mark.parametrize("budget_mb", [8, 256, 1e9])
def test_work_queue_keeps_each_pairs_order(queue_demo, budget_mb):
    """The work queue of the dataflow kernels (lcg_host::queue_order): every
    (pair, group) item once, each pair's groups in their own order, for the
    forward's small waves and the LocARNA-P backward's large ones."""
    import random
    rng = random.Random(int(budget_mb) % 1000 + 7)
    pairs = [(rng.randint(1, 3000), rng.uniform(0.5, 20) * 2 ** 20) for _ in range(300)]
    inp = f"{len(pairs)} {budget_mb * 2 ** 20}\n" + "".join(f"{g} {b}\n" for g, b in pairs)
    r = subprocess.run([queue_demo], input=inp, capture_output=True, text=True, check=True)
    word, waves = r.stdout.split()
    assert word == "ok", r.stdout
    if budget_mb == 8:
        assert int(waves) > 100
    if budget_mb == 1e9:
        assert int(waves) == 1
