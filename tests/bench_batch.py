"""Aggregate rate of the batched uneven snapshot solves (run by hand:
python tests/bench_batch.py [nsnap]).

256 snapshots (32-512 antennas in a 1 km disk, 1-8 channels in 100-200 MHz,
1-16 hour angles, 5e3-2e6 Stokes I complex64 visibilities each, image side
256-2048, cell 1/(2.2 max|uv|), epsilon 1e-5), invert + predict of every
snapshot, timed three ways on the GPU -- one plan and call sequence per
snapshot on one stream (plan creation included), the pre-planned batch on
concurrent slots, and its captured CUDA graph -- and on the CPU (the
oracle's C gridder on a sample of snapshots, scaled by visibility count).
Prints one JSON line (Mvis/s counts inverted + predicted visibilities).
"""
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import numpy  # noqa: E402
import torch  # noqa: E402


def main(nsnap=256, reps=3, cpu_sample=6):
    from rascil_gb300 import simulation as sim
    from rascil_gb300.batch import SnapshotBatch
    from rascil_gb300.wgridder import Plan
    raw = sim.snapshot_batch(nsnap)
    rng = numpy.random.default_rng(1)
    snaps, vis, models = [], [], []
    for r in raw:
        u = torch.from_numpy(r["uvw"].reshape(-1, 3) * numpy.array([-1.0, 1.0, -1.0])).cuda()
        f = torch.from_numpy(r["freq"].copy()).cuda()
        snaps.append(dict(uvw=u, freq=f, npix=r["npix"], cell=r["cell"]))
        shape = (u.shape[0], f.shape[0], 1)
        vis.append(torch.complex(torch.randn(shape, device="cuda"),
                                 torch.randn(shape, device="cuda")))
        m = torch.zeros((1, r["npix"], r["npix"]), device="cuda")
        m[0, r["npix"] // 2, r["npix"] // 2 + 3] = 1.0
        models.append(m)
    nvis = sum(r["nvis"] for r in raw)
    eps = 1e-5

    def timed(fn, n=reps):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(n):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / n

    def one_by_one():
        for i, sn in enumerate(snaps):
            p = Plan(sn["uvw"], sn["freq"], sn["npix"], sn["npix"], sn["cell"], sn["cell"], eps,
                     True, precision="fp32", grid_budget_bytes=2 << 30)
            p.ms2dirty(vis[i], layout="yx")
            p.dirty2ms(models[i], layout="yx")
            p.close()

    t_seq = timed(one_by_one, 1)
    b = SnapshotBatch(snaps, eps, precision="fp32", nslots=8)
    t_conc = timed(lambda: b.run(vis, models))
    b.capture(vis, models)
    t_graph = timed(b.replay)
    b.close()
    # CPU: the oracle's C gridder on a sample of snapshots, scaled by vis count
    from oracle import cgridder
    idx = rng.choice(nsnap, size=min(cpu_sample, nsnap), replace=False)
    cpu_t, cpu_v = 0.0, 0
    for i in idx:
        r = raw[i]
        uvw = r["uvw"].reshape(-1, 3) * numpy.array([-1.0, 1.0, -1.0])
        ms = vis[i][..., 0].cpu().numpy()
        t0 = time.perf_counter()
        cgridder.ms2dirty(uvw, r["freq"], ms, None, r["npix"], r["npix"], r["cell"], r["cell"],
                          eps, True)
        cgridder.dirty2ms(uvw, r["freq"], models[i][0].double().cpu().numpy().T, None,
                          r["cell"], r["cell"], eps, True)
        cpu_t += time.perf_counter() - t0
        cpu_v += r["nvis"]
    print(json.dumps({
        "workload": "%d snapshots, %d visibilities, image sides %s" % (
            nsnap, nvis, sorted(set(r["npix"] for r in raw))),
        "one_plan_per_snapshot_mvis_s": round(2 * nvis / t_seq / 1e6, 1),
        "batched_concurrent_mvis_s": round(2 * nvis / t_conc / 1e6, 1),
        "batched_graph_mvis_s": round(2 * nvis / t_graph / 1e6, 1),
        "seconds": {"one_plan_per_snapshot": round(t_seq, 3), "concurrent": round(t_conc, 3),
                    "graph": round(t_graph, 3)},
        "cpu_mvis_s": round(2 * cpu_v / cpu_t / 1e6, 2),
        "cpu_sample": "%d snapshots, %d visibilities, %d threads" % (
            len(idx), cpu_v, cgridder.max_threads())}))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 256)
