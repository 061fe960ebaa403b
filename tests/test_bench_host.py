"""Host-side arithmetic of bench.py's JSON line (no GPU): the whole-step
roofline of the headline step, as separate sweeps and against the fusion
floor (x read once, both outputs written once)."""
import bench


def test_headline_step_bytes():
    W = bench.WORKLOADS['mfkin128']
    # MagicFilter3D: three sweeps, each reads and writes 8 B per point;
    # Kinetic3D: 16 for the x sweep, 24 for the y and z sweeps (x and the partial sum read)
    assert W.step_bytes['sweeps'] == 3 * 16 + 16 + 24 + 24
    # x once, the two outputs once
    assert W.step_bytes['fused'] == 3 * 8
    # the dominant kernel's per-launch figure is the kinetic sweeps' mean
    assert abs(W.dom_bytes_per_pt - (16 + 24 + 24) / 3) < 1e-12


def test_step_roofline_arithmetic():
    points = 32 * 128 ** 3
    r = bench.step_roofline({'sweeps': 112.0, 'fused': 24.0}, points, 3.956e-3, 6795.1)
    assert set(r) == {'sweeps', 'fused'}
    for name, v in (('sweeps', 112.0), ('fused', 24.0)):
        gbs = v * points / 3.956e-3 / 1e9
        assert r[name]['algorithmic_bytes_per_point'] == v
        assert abs(r[name]['achieved_gbs'] - gbs) < 1e-9 * gbs
        assert abs(r[name]['frac'] - gbs / 6795.1) < 1e-12
    # the headline step measured at 3.956 ms: 1.90 TB/s as separate sweeps, 0.41 TB/s fused
    assert 0.27 < r['sweeps']['frac'] < 0.29
    assert 0.05 < r['fused']['frac'] < 0.07
