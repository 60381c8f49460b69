"""Many independent snapshot solves on one GPU.

RASCIL images a list of visibility blocks by running one invert/predict per
block through Dask (``rascil/workflows/rsexecute/imaging/imaging_rsexecute.py:
72-157``).  Here the whole list runs as one device program:

* one plan per snapshot is created up front (its w range and geometry, the
  grid oversampling from the planner's cost model: wide-field snapshots with
  few visibilities take a small oversampling, which cuts their w-plane
  transform volume several times);
* a fixed pool of workspace slots, each on its own CUDA stream, serves the
  snapshots round-robin;
* :meth:`SnapshotBatch.run_native` issues the list through ``gb_batch_run``:
  rounds in which the next batch of w-planes of every slot's snapshot is a
  job, all jobs gridded by ONE persistent launch (and degridded by one)
  that pulls (snapshot, chunk) work from a device work queue, with each
  snapshot's transforms on its slot's stream;
* the complete program (bucket sorts + invert + predict of every snapshot)
  can be captured once as a CUDA graph and replayed with a single launch.

:meth:`SnapshotBatch.run` is the same list as plain per-snapshot calls on
the slot streams (the reference for the tests).  Inputs and outputs are
preallocated device tensors so a captured graph can be replayed on new data
written into the same buffers.
"""
import torch

from .wgridder import Plan


class SnapshotBatch:
    """:param snapshots: list of dicts with device tensors ``uvw`` [R, 3]
    float64 (u, w as ng.py flips them), ``freq`` [C] float64, and ``npix``,
    ``cell``; :param nslots: concurrent workspace slots / streams (at most
    16); :param sigmas: per-snapshot grid oversampling (None: the planner's
    choice, or a cached autotuning result, per snapshot)."""

    def __init__(self, snapshots, epsilon, precision="fp32", nslots=8, do_wstacking=True,
                 device="cuda", grid_budget_bytes=2 << 30, sigmas=None):
        self.device = torch.device(device)
        self.precision = precision
        self.plans = []
        for i, sn in enumerate(snapshots):
            self.plans.append(Plan(sn["uvw"], sn["freq"], sn["npix"], sn["npix"], sn["cell"],
                                   sn["cell"], epsilon, do_wstacking, npol=1,
                                   precision=precision, bind=False,
                                   grid_budget_bytes=grid_budget_bytes,
                                   sigma=sigmas[i] if sigmas else 0.0))
        self.nslots = max(1, min(int(nslots), len(self.plans), 16))
        # slot k serves snapshots k, k + nslots, ...; size it for the largest of them
        need = [0] * self.nslots
        for i, p in enumerate(self.plans):
            need[i % self.nslots] = max(need[i % self.nslots], p.workspace_bytes)
        self.workspaces = [torch.empty(max(n, 256), dtype=torch.uint8, device=self.device)
                           for n in need]
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(self.nslots)]
        cdt = self.plans[0].complex_dtype if self.plans else torch.complex64
        rdt = self.plans[0].real_dtype if self.plans else torch.float32
        self.dirty = [torch.empty((1, p.npix_y, p.npix_x), dtype=rdt, device=self.device)
                      for p in self.plans]
        self.pred = [torch.empty((p.nrows, p.nchan, 1), dtype=cdt, device=self.device)
                     for p in self.plans]
        self.graph = None

    @property
    def nvis(self):
        return sum(p.nrows * p.nchan for p in self.plans)

    def run(self, vis, models, concurrent=True):
        """Invert vis[i] into self.dirty[i] and predict models[i] into
        self.pred[i] for every snapshot, on the current stream's timeline."""
        main = torch.cuda.current_stream(self.device)
        streams = self.streams if concurrent else [main] * self.nslots
        if concurrent:
            for s in streams:
                s.wait_stream(main)
        for i, p in enumerate(self.plans):
            k = i % self.nslots
            with torch.cuda.stream(streams[k]):
                p.bind(self.workspaces[k])
                p.ms2dirty(vis[i], layout="yx", out=self.dirty[i])
                p.dirty2ms(models[i], layout="yx", out=self.pred[i])
        if concurrent:
            for s in streams:
                main.wait_stream(s)

    def run_native(self, vis, models):
        """run(vis, models) as one device program (``gb_batch_run``): rounds
        over the slots' current snapshots, each round's gridding and
        degridding of every snapshot in one persistent launch fed from a
        device work queue, the transforms on the slot streams; no Python
        round trip per snapshot."""
        import ctypes

        from . import _lib
        n = len(self.plans)
        if len(vis) != n or len(models) != n:
            raise ValueError("one vis and one model per snapshot")
        for i, p in enumerate(self.plans):
            v, m = vis[i], models[i]
            if (not v.is_cuda or v.dtype != p.complex_dtype or not v.is_contiguous()
                    or v.numel() != p.nrows * p.nchan * p.npol):
                raise ValueError("vis[%d] must be a contiguous %s CUDA tensor of %d values"
                                 % (i, p.complex_dtype, p.nrows * p.nchan * p.npol))
            if (not m.is_cuda or m.dtype != p.real_dtype or not m.is_contiguous()
                    or m.numel() != p.npol * p.npix_x * p.npix_y):
                raise ValueError("models[%d] must be a contiguous %s CUDA tensor of %d values"
                                 % (i, p.real_dtype, p.npol * p.npix_x * p.npix_y))
        main = torch.cuda.current_stream(self.device)
        for s in self.streams:
            s.wait_stream(main)
        ptrs = ctypes.c_void_p * n
        slots = ctypes.c_void_p * self.nslots
        args = (ptrs(*[p._handle.value for p in self.plans]), n,
                slots(*[w.data_ptr() for w in self.workspaces]),
                (ctypes.c_size_t * self.nslots)(*[w.numel() for w in self.workspaces]),
                slots(*[s.cuda_stream for s in self.streams]), self.nslots,
                ptrs(*[t.data_ptr() for t in vis]), ptrs(*[t.data_ptr() for t in self.dirty]),
                ptrs(*[t.data_ptr() for t in models]), ptrs(*[t.data_ptr() for t in self.pred]),
                _lib.GB_LAYOUT_YX)
        with torch.cuda.device(self.device):
            _lib.check(_lib.load().gb_batch_run(*args), "gb_batch_run")
        for i, p in enumerate(self.plans):
            p.workspace = self.workspaces[i % self.nslots]
        for s in self.streams:
            main.wait_stream(s)

    def capture(self, vis, models, native=True):
        """Record run_native(vis, models) (or run() with native=False) as a
        CUDA graph; replay() re-runs it."""
        fn = self.run_native if native else self.run
        fn(vis, models)  # warm-up outside capture (cuFFT, caches)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            fn(vis, models)
        self.graph = g
        self._keep = (vis, models)
        return g

    def replay(self):
        if self.graph is None:
            raise RuntimeError("capture() first")
        self.graph.replay()

    def close(self):
        torch.cuda.synchronize(self.device)
        for p in self.plans:
            p.close()
        self.plans = []
        self.graph = None
