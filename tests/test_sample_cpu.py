"""The ray-sample checker (oracle/sample.py) on the CPU: with every ray sampled its sample
spectrum is the oracle's own image -> F_nu sum; the error measures behave as stated."""
import numpy as np

PC2 = 3.08572e18 ** 2


def test_full_sample_is_the_spectrum(oracle_lib, model_dir):
    from oracle import sample
    d = model_dir("tiny_line")
    o = oracle_lib.Oracle(d)
    rows, counts, _, _ = sample.oracle_rows(d, [o.ilinestart], np.arange(o.nrays), procs=2)
    img, _, cnt = o.line_image(o.ilinestart)
    np.testing.assert_array_equal(rows[0], img)
    assert counts[1] == cnt["integrated"] and counts[0] == cnt["steps"]
    _, _, _, ri = o.rays()
    spec = sample.sample_spectrum(rows, np.arange(o.nrays), ri, o.nphi)[0] / PC2
    ref, _, _ = o.line_spectrum(o.ilinestart)
    np.testing.assert_allclose(spec, ref, rtol=1e-12, atol=0)


def test_error_measures():
    from oracle import sample
    ref = np.array([[1.0, 2.0, 4.0], [0.0, 0.0, 0.0]])
    got = ref.copy()
    got[0, 1] += 4e-4
    assert abs(sample.pixel_relerr(got, ref) - 1e-4) < 1e-15
    assert sample.pixel_relerr(np.zeros((1, 2)), np.zeros((1, 2))) == 0.0
    assert sample.pixel_relerr(np.ones((1, 2)), np.zeros((1, 2))) == float("inf")
    assert abs(sample.spectrum_relerr(np.array([1.0, 2.0002]), np.array([1.0, 2.0])) - 1e-4) < 1e-12
    assert list(sample.ray_sample(10, 4, 1)) == [1, 5, 9]
