"""GPU batched path: many per-group trees, one persistent density launch (optionally a
replayed CUDA graph), autotuned leaf / query-bucket sizes; checked per group against the
oracle's KDTree(group) + CalcDensity(min(k, n-1)) and against the per-tree loop."""
import concurrent.futures as cf
import json
import os

import numpy as np
import pytest

import oracle
from nbodylib_gb300 import BatchedDensity
from nbodylib_gb300 import synthetic as syn
from tests.helpers import assert_density_close

pytestmark = pytest.mark.gpu


def reference_batch(pos, mass, off, k, b, threads=1):
    """The reference's per-group pattern on the restatement: KDTree(group) +
    CalcDensity(min(k, n - 1)) for every group (groups spread over host threads)."""
    rho = np.empty(len(mass))

    def one(g):
        s, e = int(off[g]), int(off[g + 1])
        if e - s < 2:
            rho[s:e] = 0.0
            return
        t = oracle.OracleTree(pos[s:e], None, mass[s:e], b, 0, 0, 1000, None, backend="port",
                              nthreads=1)
        rho[s:e] = t.density(min(k, e - s - 1))
        t.close()

    if threads <= 1:
        for g in range(len(off) - 1):
            one(g)
    else:
        with cf.ThreadPoolExecutor(threads) as ex:
            list(ex.map(one, range(len(off) - 1)))
    return rho


@pytest.mark.parametrize("bucket", [16, 0])
def test_batched_density_vs_oracle(gpu, port_built, bucket):
    sizes = syn.group_sizes(300, 20, 3000, seed=41)
    sizes[:3] = [2, 3, 33]  # tiny groups: k is clamped to n - 1
    pos, vel, mass, off = syn.plummer_groups(sizes, seed=41)
    want = reference_batch(pos, mass, off, 32, 16)
    B = BatchedDensity(pos, mass, off, bucket_size=bucket)
    b, qb, tune = B.params()
    if bucket == 0:
        assert b in (8, 12, 16, 24, 32) and qb in (16, 32) and "chosen" in tune
        tune = json.loads(tune)
        # every (leaf size, query bucket, query mapping) candidate was timed
        assert len(tune["median_ms_build_search"]) == 5 * 2 * 2
        assert tune["chosen"]["warp_per_query"] == B.query_mapping()
    for wpq in (1, 0):
        B.set_query_mapping(wpq)
        for use_graph in (False, True, True):
            assert_density_close(B.density(32, use_graph=use_graph), want,
                                 f"batched graph={use_graph} warp_per_query={wpq}")
    assert_density_close(B.density_pertree(32), want, "per-tree loop")
    assert_density_close(B.density_pertree_search(32), want, "per-tree search loop")
    B.close()


def test_batched_graph_on_caller_stream(gpu, port_built):
    """A graph captured and replayed on a caller's torch stream gives the same density
    as the host-array path, for device-resident inputs."""
    import torch
    sizes = syn.group_sizes(200, 20, 2000, seed=44)
    pos, vel, mass, off = syn.plummer_groups(sizes, seed=44)
    want = reference_batch(pos, mass, off, 32, 16)
    st = torch.cuda.Stream()
    B = BatchedDensity(torch.from_numpy(pos).cuda(), torch.from_numpy(mass).cuda(),
                       torch.from_numpy(off).cuda(), bucket_size=16, device=True)
    B.set_stream(st)
    rho = torch.empty(len(mass), dtype=torch.float64, device="cuda")
    for _ in range(3):
        B.density(32, use_graph=True, out=rho)
    st.synchronize()
    assert_density_close(rho.cpu().numpy(), want, "graph on caller stream")
    B.close()


def test_batched_large_groups(gpu, port_built):
    """Groups above the 1024-particle per-CTA limit go through the level-synchronous
    phase together."""
    sizes = np.array([5000, 1025, 70000, 20, 4096, 1500])
    pos, vel, mass, off = syn.plummer_groups(sizes, seed=43)
    want = reference_batch(pos, mass, off, 32, 16)
    B = BatchedDensity(pos, mass, off, bucket_size=16)
    assert_density_close(B.density(32), want, "large groups")


def test_batched_density_full_powerlaw_batch(gpu, port_built):
    """The benchmarked batch itself: 20,000 Plummer groups with sizes n^-2 on
    [20, 200000] (3,657,291 particles), k = min(32, n - 1), every density against the
    restatement's per-group KDTree + CalcDensity, through the replayed graph with the
    plain leaf size and with the autotuned one, and through the per-tree loop."""
    sizes = syn.group_sizes(20000, 20, 200000, seed=4)
    pos, vel, mass, off = syn.plummer_groups(sizes, seed=4)
    assert len(mass) == 3657291
    want = reference_batch(pos, mass, off, 32, 16, threads=os.cpu_count() or 1)
    for bucket in (16, 0):
        B = BatchedDensity(pos, mass, off, bucket_size=bucket)
        b, qb, _ = B.params()
        for _ in range(2):
            assert_density_close(B.density(32, use_graph=True), want,
                                 f"full batch, b={b} qb={qb}, graph")
        if bucket == 16:
            assert_density_close(B.density_pertree_search(32), want, "full batch, per-tree")
        B.close()
