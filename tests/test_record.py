"""Run directory of the recorder: every dataset written is read back in
the reference's layout ([output][bunch][...]), and the resume state is the
last saved phase space."""
import numpy as np

from inovesa_gb300 import record as R


def test_recorder_roundtrip(tmp_path):
    n, nb = 16, 2
    rec = R.Recorder(str(tmp_path), np.linspace(-6, 6, n),
                     np.linspace(-6, 6, n), np.arange(32.0), buckets=(0, 3),
                     ps_every=2)
    rng = np.random.default_rng(0)
    saved = []
    for k in range(5):
        ps = rng.random((nb, n, n), dtype=np.float32)
        saved.append(ps)
        rec.append(0.1 * k, np.ones(nb), rng.random((nb, n)),
                   rng.random((nb, n)), rng.random(nb), rng.random(nb),
                   rng.random(nb), rng.random(nb), rng.random((nb, n)),
                   rng.random((nb, 32)), rng.random(nb), ps)
    rec.close()
    assert R.read(str(tmp_path), "/BunchProfile/data").shape == (5, nb, n)
    assert R.read(str(tmp_path), "/CSR/Spectrum/data").shape == (5, nb, 32)
    assert np.array_equal(R.read(str(tmp_path), "/Info/BucketNumbers"),
                          [0, 3])
    # phase space every 2nd output: outputs 0, 2, 4
    psd = R.read(str(tmp_path), "/PhaseSpace/data")
    assert psd.shape == (3, nb, n, n)
    state, t = R.resume_state(str(tmp_path))
    assert np.array_equal(state, saved[4]) and abs(t - 0.4) < 1e-12
