"""Shared checks of the GPU parity tests."""
import numpy as np

# Per-move scores: FP32 kernel vs FP64 oracle, relative to the local score
# scale of the move (max(|before|, |after|, 1e-3)).
LOCAL_TOL = 1e-5
# A kernel decision may differ from the oracle's only when the move sat this
# close to the Metropolis threshold (|ln(E_new/E_prev) - ln(ratio threshold)|).
MARGIN_TOL = 1e-4


def check_replay(trace, rep, scale_factor=1.0, delta_only=False):
    ob = rep["before"]
    oa = rep["after"]
    scale = np.maximum(np.maximum(np.abs(ob), np.abs(oa)), 1e-3) * scale_factor
    if delta_only:
        err = np.abs(trace["after"].astype(np.float64) - scale_factor * (oa - ob)) / scale
    else:
        err = np.maximum(np.abs(trace["before"] - ob), np.abs(trace["after"] - oa)) / scale
    assert rep["proposal_mismatch"] == 0, "Philox proposals differ from the oracle's"
    assert err.max() <= LOCAL_TOL, f"local score error {err.max():.3g} at move {err.argmax()}"
    mism = trace["accepted"] != rep["orc_acc"]
    if mism.any():
        assert rep["margin"][mism].max() < MARGIN_TOL, \
            f"decision mismatch far from threshold: {rep['margin'][mism].max():.3g}"
    assert mism.sum() <= max(2, len(trace) // 1000)
    return err.max(), int(mism.sum())


def kabsch_rmsd(a, b):
    a = a - a.mean(0)
    b = b - b.mean(0)
    h = a.T @ b
    u, s, vt = np.linalg.svd(h)
    d = np.sign(np.linalg.det(vt.T @ u.T))
    m = np.diag([1.0, 1.0, d])
    r = vt.T @ m @ u.T
    return float(np.sqrt(((a @ r.T - b) ** 2).sum(1).mean()))


def distmap_pearson(a, b):
    iu = np.triu_indices(len(a), 1)
    da = np.linalg.norm(a[:, None] - a[None], axis=2)[iu]
    db = np.linalg.norm(b[:, None] - b[None], axis=2)[iu]
    return float(np.corrcoef(da, db)[0, 1])


def ks_2samp_p(x, y):
    from scipy import stats
    return float(stats.ks_2samp(x, y).pvalue)


def welch_p(x, y):
    """Two-sided Welch t-test p-value (equal means, unequal variances)."""
    from scipy import stats
    return float(stats.ttest_ind(x, y, equal_var=False).pvalue)
