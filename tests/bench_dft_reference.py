"""Time the GPU component DFT against the reference's own CUDA kernel on the
same GPU and inputs (run by hand: python tests/bench_dft_reference.py).

Workload: the LOW-like geometry (130,816 baselines), 2 hour angles, 16
channels 100-200 MHz, 4 linear polarisations, its 1,000 point sources;
FP64 in both.  Prints one JSON line.
"""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import numpy  # noqa: E402
import torch  # noqa: E402


def main(ntimes=2):
    from oracle import ref_dft
    from rascil_gb300 import simulation as sim
    from rascil_gb300.dft import dft_components
    uvw, freq, pc, cfg = sim.observation("low-like", ntimes=ntimes)
    src = sim.sources(cfg)
    lmn = sim.lmn_rows(src)
    flux = sim.component_fluxes(cfg, src, len(freq))
    u = torch.from_numpy(uvw.reshape(-1, 3).copy()).cuda()
    f = torch.from_numpy(freq.copy()).cuda()
    uvw_lambda = (torch.from_numpy(uvw).cuda()[:, :, None, :]
                  * (f / 299792458.0)[None, None, :, None]).contiguous()
    lmn_t = torch.from_numpy(lmn).cuda().contiguous()
    flux_t = torch.from_numpy(flux).cuda().contiguous()
    ref = torch.zeros(uvw.shape[:2] + (len(freq), flux.shape[-1]), dtype=torch.complex128,
                      device="cuda")

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            out = fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps, out

    t_ref, _ = timed(lambda: ref_dft.run(lmn_t, flux_t, uvw_lambda, ref))
    t_ours, ours = timed(lambda: dft_components(u, f, lmn, flux, precision="fp64", exact=True))
    t_fast, fast = timed(lambda: dft_components(u, f, lmn, flux, precision="fp32", exact=False))
    b = ref.cpu().numpy()
    a = ours.reshape(ref.shape).cpu().numpy()
    c = fast.reshape(ref.shape).cpu().numpy().astype(numpy.complex128)
    nvis = b.size
    print(json.dumps({
        "workload": "LOW-like geometry, %d times x %d baselines x %d chan x %d pol, %d components"
                    % (ntimes, uvw.shape[1], len(freq), flux.shape[-1], len(lmn)),
        "reference_dft_kernel_ms": round(t_ref, 3),
        "gb_dft_exact_fp64_ms": round(t_ours, 3),
        "gb_dft_fast_ms": round(t_fast, 3),
        "speedup_exact": round(t_ref / t_ours, 2),
        "speedup_fast": round(t_ref / t_fast, 2),
        "max_rel_diff_exact": float(numpy.max(numpy.abs(a - b)) / numpy.max(numpy.abs(b))),
        "rel_rms_fast": float(numpy.linalg.norm(c - b) / numpy.linalg.norm(b)),
        "vis_comp_pairs_per_s_exact": nvis / flux.shape[-1] * len(lmn) / (t_ours * 1e-3)}))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 2)
