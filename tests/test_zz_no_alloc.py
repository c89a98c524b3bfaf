"""rl_image_to_spectrum_noalloc: the reduction that keeps its ring sums in a fixed array of
the library instead of allocating. Its spectra must equal those of rl_spectra, the
regular entry point, on the same circular images, call after call.

Tolerances: an FP64 image gives the regular path's sum up to the order of one multiply
(<= 1e-12 relative); an FP32 copy of the image adds its own rounding (<= 1e-6)."""
import ctypes as C

import numpy as np
import pytest

FP64_TOL = 1e-12
FP32_TOL = 1e-6


def _call(rl, stream, prec, img, nlines, nrays, nphi, nrr, nfr, ri, scale, flux):
    return rl.lib().rl_image_to_spectrum_noalloc(stream, prec, img, nlines, nrays, nphi, nrr, nfr, ri, scale,
                                                 1.0, flux)


def test_rejects_bad_sizes_before_touching_memory(gpu_lib):
    rl = gpu_lib
    fake = C.c_void_p(256)   # never dereferenced: every case below fails the host checks
    # ring sums beyond the fixed 2^20-double scratch
    rc = _call(rl, None, 0, fake, 1, 1 + 2048 * 4, 4, 2048, 600, fake, fake, fake)
    assert rc == -1
    assert "fixed scratch" in rl._err()
    rc = _call(rl, None, 0, fake, 1, 100, 4, 10, 50, fake, fake, fake)   # nrays != 1 + nrr*nphi
    assert rc == -1 and "1 + nrr * nphi" in rl._err()
    rc = _call(rl, None, 2, fake, 1, 41, 4, 10, 50, fake, fake, fake)
    assert rc == -1 and "precision" in rl._err()
    rc = _call(rl, None, 0, None, 1, 41, 4, 10, 50, fake, fake, fake)
    assert rc == -1 and "null" in rl._err()


@pytest.mark.gpu
def test_noalloc_matches_regular_entry_point(gpu_lib, oracle_lib, model_dir):
    import torch
    rl = gpu_lib
    d = model_dir("tiny_band")
    ctx = rl.Context(0)
    m = ctx.load_dir(d)
    info = m.info()
    il0, nl, nfr = info["ilinestart"], info["nlines_spec"], info["nfr"]
    nrays, nphi = info["nrays"], info["nphi"]
    nrr = (nrays - 1) // nphi
    regular = m.spectra(il0, nl)                                       # [nl, nfr]
    images = np.stack([m.line_image(il0 + k) for k in range(nl)])      # scaled intensities
    _, _, _, ri = oracle_lib.Oracle(d).rays()                          # ring edges of this camera
    assert ri.shape == (nrr + 2,)
    dev = torch.device("cuda", 0)
    img64 = torch.from_numpy(images).to(dev)
    img32 = img64.float()
    dri = torch.from_numpy(ri).to(dev)
    ones = torch.ones(nl, dtype=torch.float64, device=dev)
    flux = torch.full((nl, nfr), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize(dev)
    for call in range(2):
        for prec, img, tol in ((1, img64, FP64_TOL), (0, img32, FP32_TOL)):
            flux.fill_(float("nan"))
            rc = _call(rl, stream, prec, img.data_ptr(), nl, nrays, nphi, nrr, nfr, dri.data_ptr(),
                       ones.data_ptr(), flux.data_ptr())
            assert rc == 0, rl._err()
            got = flux.cpu().numpy()
            for k in range(nl):
                ref = regular[k]
                sel = ref > 1e-3 * ref.max()
                rel = np.max(np.abs(got[k][sel] - ref[sel]) / np.abs(ref[sel]))
                assert rel <= tol, (call, prec, k, rel)
    # the call allocates nothing: the device's free memory is unchanged across a call. Free
    # memory is device-wide, so another process can move it; one unchanged attempt of a few
    # is enough.
    unchanged = False
    for _ in range(5):
        torch.cuda.synchronize(dev)
        free0 = torch.cuda.mem_get_info(dev)[0]
        rc = _call(rl, stream, 1, img64.data_ptr(), nl, nrays, nphi, nrr, nfr, dri.data_ptr(), ones.data_ptr(),
                   flux.data_ptr())
        assert rc == 0, rl._err()
        torch.cuda.synchronize(dev)
        if torch.cuda.mem_get_info(dev)[0] == free0:
            unchanged = True
            break
    assert unchanged
    m.free()
    ctx.close()


@pytest.mark.gpu
def test_noalloc_line_chunks(gpu_lib):
    """Lines whose ring sums do not fit the scratch together are reduced in chunks."""
    import torch
    rl = gpu_lib
    nrr, nphi, nfr, nl = 1100, 8, 700, 3          # (nrr+1)*nfr = 770700: one line per chunk
    nrays = 1 + nrr * nphi
    rng = np.random.default_rng(7)
    img = rng.random((nl, nrays, nfr))
    ri = np.concatenate([[0.0], np.cumsum(rng.random(nrr + 1) + 0.5)])
    scale = np.array([1.0, 2.5, 0.25])
    dev = torch.device("cuda", 0)
    dimg, dri, dsc = (torch.from_numpy(a).to(dev) for a in (img, ri, scale))
    flux = torch.zeros((nl, nfr), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize(dev)
    rc = _call(rl, stream, 1, dimg.data_ptr(), nl, nrays, nphi, nrr, nfr, dri.data_ptr(), dsc.data_ptr(),
               flux.data_ptr())
    assert rc == 0, rl._err()
    got = flux.cpu().numpy()
    pc = 3.08572e18
    area = np.pi * np.diff(ri[1:] ** 2)                                       # rings 1..nrr
    rings = img[:, 1:, :].reshape(nl, nrr, nphi, nfr).mean(axis=2)
    ref = (np.pi * ri[1] ** 2 * img[:, 0, :] + np.einsum("r,lrf->lf", area, rings)) * scale[:, None] / pc ** 2
    np.testing.assert_allclose(got, ref, rtol=1e-12)
