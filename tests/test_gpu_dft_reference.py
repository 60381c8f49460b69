"""The GPU component DFT against the reference's own CUDA kernel
(rascil/processing_components/imaging/dft.py:181-258), compiled from the
reference tree by oracle/ref_dft, on the same inputs."""
import numpy
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_component_dft_matches_reference_cuda_kernel():
    from oracle import ref_dft
    if not ref_dft.available():
        pytest.skip("reference kernel source not extracted (no reference tree at build time)")
    from rascil_gb300 import simulation as sim
    from rascil_gb300.dft import dft_components
    uvw, freq, pc, cfg = sim.observation("low-like", ntimes=2, nchan=5, nants=64)
    cfg["nsrc"] = 37
    src = sim.sources(cfg)
    lmn = sim.lmn_rows(src)
    flux = sim.component_fluxes(cfg, src, len(freq))
    u = torch.from_numpy(uvw.reshape(-1, 3).copy()).cuda()
    f = torch.from_numpy(freq.copy()).cuda()
    ours = dft_components(u, f, lmn, flux, precision="fp64", exact=True)
    uvw_lambda = (torch.from_numpy(uvw).cuda()[:, :, None, :]
                  * (f / 299792458.0)[None, None, :, None]).contiguous()
    ref = torch.zeros(uvw.shape[:2] + (len(freq), flux.shape[-1]), dtype=torch.complex128,
                      device="cuda")
    ref_dft.run(torch.from_numpy(lmn).cuda().contiguous(),
                torch.from_numpy(flux).cuda().contiguous(), uvw_lambda, ref)
    torch.cuda.synchronize()
    a = ours.reshape(ref.shape).cpu().numpy()
    b = ref.cpu().numpy()
    assert numpy.max(numpy.abs(a - b)) < 1e-11 * numpy.max(numpy.abs(b))
