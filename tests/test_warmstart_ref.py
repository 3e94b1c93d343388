"""The numpy restatement of the warm-start network (the checker of the GPU
gradients) against central finite differences."""
import numpy as np

from oracle import warmstart_ref as R


def test_reference_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    nin, nh, nlat, npix, B = 3, 7, 4, 11, 5
    w = {"w1": rng.normal(size=(nh, nin)), "b1": rng.normal(size=nh),
         "w2": rng.normal(size=(nh, nh)) / 3, "b2": rng.normal(size=nh),
         "w3": rng.normal(size=(nlat, nh)), "b3": rng.normal(size=nlat),
         "wd": rng.normal(size=(nlat, npix)), "bd": rng.normal(size=npix)}
    x = rng.normal(size=(B, nin))
    t = rng.normal(size=(B, npix))
    _, g = R.loss_and_grads(w, x, t)
    eps = 1e-6
    for k, v in w.items():
        flat = v.reshape(-1)
        for i in rng.choice(flat.size, size=min(6, flat.size), replace=False):
            old = flat[i]
            flat[i] = old + eps
            lp, _ = R.loss_and_grads(w, x, t)
            flat[i] = old - eps
            lm, _ = R.loss_and_grads(w, x, t)
            flat[i] = old
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - g[k].reshape(-1)[i]) <= 1e-6 * max(1, abs(fd)), k
