"""The device-side noise stream (bd_dev_noise_*) against the host stream
(bd_noise_step, which the CPU tests pin to the reference's mt.cpp and
utilities.cpp).  Same seed, same sequence of steps: every deviate equal bit
for bit to a host stream set to the correctly rounded log (BD_LOG_CR, the
device's), and to the reference's host stream (the C library's log) except
where that log rounds differently (last bits, well under 1% of the
deviates); the generators stay in step across LH Monte-Carlo steps
(step % 100 == 0), cached deviates (odd draw counts) and many twists per
step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n3,nD3", [(111, 3003), (3 * 96, 3 * 1296), (30, 40001)])
def test_device_stream_matches_host(n3, nD3):
    import torch
    from brownian_dynamics_cuda_gb300 import LOG_CR, DevNoise, Noise
    r_var = np.abs(np.random.default_rng(n3).normal(size=n3)) + 0.1
    host, dev = Noise(42), DevNoise(42)
    cr = Noise(42, log_mode=LOG_CR)
    d_rvar = torch.tensor(r_var, dtype=torch.float64, device="cuda")
    d_rr = torch.empty(n3, dtype=torch.float64, device="cuda")
    d_p = torch.empty(nD3, dtype=torch.float64, device="cuda")
    exact = total = 0
    for step in (0, 1, 2, 99, 100, 101, 200, 201, 202, 203):
        rr_h, p_h = host.step(step, r_var, nD3)
        rr_c, p_c = cr.step(step, r_var, nD3)
        dev.step(step, d_rvar.data_ptr(), n3, nD3, d_rr.data_ptr(), d_p.data_ptr())
        torch.cuda.synchronize()
        for h, c, d in ((rr_h, rr_c, d_rr.cpu().numpy()), (p_h, p_c, d_p.cpu().numpy())):
            assert np.array_equal(d, c), (step, int(np.sum(d != c)))
            assert np.all(np.abs(d - h) <= 4 * np.spacing(np.abs(h))), (step, np.max(np.abs(d - h) / np.abs(h)))
            exact += int(np.sum(d == h))
            total += h.size
    assert exact >= 0.99 * total
