"""The bench line's kernel table (bench.kernel_table) on a synthetic trace: the
per-kernel rates, the paint-stage and FFT-stage aggregates, and no byte model
for the recount and fill launches that return at once with bucketed lists."""
import pytest

import bench


def _trace(steps):
    # ms per launch of a 512^3-particle / 1024^3-mesh TSC step (one force each)
    per = {'kick_drift_bin': 2.818, 'paint_bin_count': 0.015, 'paint_bin_scan': 0.012,
           'paint_bin_fill': 0.010, 'paint_tsc': 3.352, 'fft_z_r2c': 1.520, 'fft_y_fwd': 1.987,
           'fft_x_fwd_transfer_inv': 3.408, 'fft_y_inv': 1.998, 'fft_z_c2r': 1.646,
           'grad_stencil': 4.895, 'readout4_tsc': 6.234}
    return {k: (steps, v * steps) for k, v in per.items()}


@pytest.mark.parametrize('bucketed', [True, False])
def test_kernel_table_stages(bucketed):
    n, np_ = 1024, 512 ** 3
    alg = bench.algorithmic_bytes(n, np_, 'tsc', stencil=True, packed=True)
    kern = _trace(40)
    k = bench.kernel_table(kern, alg, 6778.0, 40, 'tsc', bucketed)
    # the readout: 16 M + 28 Np bytes per launch
    assert k['readout4_tsc']['gbs'] == pytest.approx((16 * n ** 3 + 28 * np_) / 6.234e-3 / 1e9)
    # the paint stage: 12 Np + 4 M bytes over the scan, recount, fill and deposit
    t = 3.352 + 0.015 + 0.012 + 0.010
    assert k['paint_stage']['ms_per_launch'] == pytest.approx(t)
    assert k['paint_stage']['frac'] == pytest.approx((12 * np_ + 4 * n ** 3) / t / 1e6 / 6778.0)
    # the FFT stage: the five passes of one force
    ffts = ['fft_z_r2c', 'fft_y_fwd', 'fft_x_fwd_transfer_inv', 'fft_y_inv', 'fft_z_c2r']
    assert sorted(k['fft_stage']['kernels']) == sorted(ffts)
    assert k['fft_stage']['ms_per_launch'] == pytest.approx(sum(kern[f][1] for f in ffts) / 40)
    assert 0.55 < k['fft_stage']['frac'] < 0.65
    for name in ('paint_bin_count', 'paint_bin_fill'):
        if bucketed:
            assert 'frac' not in k[name] and 'note' in k[name]
        else:
            assert 'frac' in k[name]
    shares = sum(v['share'] for name, v in k.items() if not name.endswith('_stage'))
    assert shares == pytest.approx(1.0)
