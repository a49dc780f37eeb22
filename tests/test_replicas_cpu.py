"""The multi-GPU plan's host side over two `gloo` ranks on CPU (no GPU): frames and views dealt
round-robin over the ranks, timings reduced to the slowest rank, and the differentiable
renderer's parameter gradients summed over views rendered on different ranks, which must equal
the gradients of all views computed in one process (the FP64 oracle computes each view's part)."""
import datetime
import os
import socket

import numpy as np
import pytest

from dfpsr_gb300 import replicas, scenes

VIEWS = 4


def _problem():
    return scenes.diff_problem(seed=3, views=VIEWS, size=32, texture_size=16, major=12, minor=8)


def _view_gradients(problem, view):
    """Parameter gradients of one view's L2 loss on a seeded visibility buffer (FP64 oracle)."""
    from oracle import diff64
    rng = np.random.default_rng(100 + view)
    slots = diff64.fan_triangles(problem.mesh.poly_indices)
    vis = np.zeros((2000, 3), np.uint32)
    vis[:, 0] = rng.integers(0, len(slots), size=len(vis))
    b = rng.uniform(0, 1, size=len(vis)).astype(np.float32)
    c = (rng.uniform(0, 1, size=len(vis)) * (1 - b)).astype(np.float32)
    vis[:, 1] = b.view(np.uint32)
    vis[:, 2] = c.view(np.uint32)
    vis[rng.uniform(size=len(vis)) < 0.2, 0] = diff64.NO_TRIANGLE
    shading = diff64.Shading(problem.mesh, vis, problem.texture.shape)
    targets = rng.uniform(0, 1, size=(len(vis), 4))
    out, _ = shading.forward(problem.texture, problem.vertex_colors, problem.light, problem.ambient)
    return shading.gradients(problem.texture, problem.vertex_colors, problem.light, problem.ambient, diff64.l2_grad(out, targets))


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=60))
    try:
        frames = replicas.my_units(10, rank, world)
        slowest = replicas.max_over_ranks(1.5 + rank, dist)
        problem = _problem()
        local = None
        for v in replicas.my_units(VIEWS, rank, world):
            g = _view_gradients(problem, v)
            local = list(g) if local is None else [a + b for a, b in zip(local, g)]
        summed = replicas.sum_over_ranks(local, dist)
        gathered = replicas.gather_on_root(frames, dist)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), frames=np.array(frames), slowest=slowest,
                 texture=summed[0], vertex_colors=summed[1], light=summed[2],
                 gathered=np.array(gathered if gathered is not None else [], dtype=object), allow_pickle=True)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_units_are_dealt_round_robin():
    assert replicas.my_units(7, 0, 3) == [0, 3, 6]
    assert replicas.my_units(7, 2, 3) == [2, 5]
    assert sorted(sum((replicas.my_units(11, r, 4) for r in range(4)), [])) == list(range(11))
    with pytest.raises(ValueError):
        replicas.my_units(4, 2, 2)
    # without a process group every helper is the single-rank identity
    assert replicas.max_over_ranks(2.5) == 2.5
    a = np.arange(6.0).reshape(2, 3)
    assert np.array_equal(replicas.sum_over_ranks([a])[0], a)
    assert replicas.gather_on_root("x") == ["x"]


def test_two_gloo_ranks_split_frames_and_sum_view_gradients(tmp_path, built):
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    spawn = mp.get_context("spawn")
    procs = [spawn.Process(target=_rank_main, args=(r, world, port, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    for p in procs:
        if p.is_alive():
            p.kill()
            p.join()
    assert [p.exitcode for p in procs] == [0] * world
    res = [np.load(os.path.join(tmp_path, f"rank{r}.npz"), allow_pickle=True) for r in range(world)]
    assert sorted(np.concatenate([r["frames"] for r in res]).tolist()) == list(range(10))
    assert all(float(r["slowest"]) == 2.5 for r in res)
    assert [list(x) for x in res[0]["gathered"]] == [[0, 2, 4, 6, 8], [1, 3, 5, 7, 9]]
    # the views' gradients summed across ranks equal those of all views in one process
    problem = _problem()
    whole = None
    for v in range(VIEWS):
        g = _view_gradients(problem, v)
        whole = list(g) if whole is None else [a + b for a, b in zip(whole, g)]
    for r in res:
        for name, expect in zip(("texture", "vertex_colors", "light"), whole):
            np.testing.assert_allclose(r[name], expect, rtol=1e-12, atol=1e-15)
    assert np.array_equal(res[0]["texture"], res[1]["texture"])
