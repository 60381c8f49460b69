"""CPU oracle for the w-stacking gridder -- TEST INFRASTRUCTURE ONLY.

Nothing in the product (``rascil_gb300``) imports this package.  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg (``--impl reference`` and the ``cpu_baseline`` object) use it, and
only as the checker or as the timed CPU stand-in for the reference.

Contents
--------
``dft``        FP64 direct transforms: the point-source DFT of
               ``rascil/processing_components/imaging/dft.py:261-281``
               (``dft_cpu_looped``) and the exact image-plane operator
               that ``ducc0.wgridder.ms2dirty`` / ``dirty2ms`` approximate
               (call sites ``rascil/processing_components/imaging/ng.py:91-120,
               232-275``).
``wgridder``   FP64 numpy restatement of the w-stacking exponential-of-
               semicircle gridder (the published algorithm of ducc0 0.24.0,
               which is a pip dependency absent from the reference tree):
               same planning, bucketing and correction as the CUDA path.
``cgridder``   ctypes wrapper of ``wgridder.c``: the same algorithm in
               multithreaded C, used as the timed CPU baseline.

Parity status: the point-source DFT is pinned against golden vectors made
by running the reference's own ``dft_cpu_looped`` and polarisation code
(``tests/golden/make_golden.py``); the image-plane operator is pinned by
the reference's configuration-independent known answers (centre pixel
predicts V = 1, PSF peak = 1, ``tests/processing_components/
test_imaging.py:274-293,601-611``).  ducc0 itself cannot be run here, so
bit-level parity with ducc0's own output is unpinned.
"""
