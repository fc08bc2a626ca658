"""PPHPC focal measures and the two-sample comparison used to check that two
implementations of the model are statistically indistinguishable.

The outputs of one run are the six per-iteration series of the stats file
(opencl/pp/pp_common.c:205-240): sheep count, wolf count, live-grass count,
mean sheep energy, mean wolf energy and mean grass countdown. The focal
measures of a series X[0..iters] (Fachada et al., "Towards a standard model
for research in agent-based modeling and simulation", PeerJ CS 2015) are

    max X, argmax X, min X, argmin X,
    mean and sample std of X over the steady state (iterations > ss_from).

For each measure the replications of the two implementations form two
samples. They are compared as in that paper: when both samples pass the
Shapiro-Wilk normality test, with Welch's t-test; otherwise with the
Mann-Whitney U test. A measure that is constant and equal in both samples
counts as equal. The family of p-values is corrected with Holm's step-down
method, so `alpha` is the family-wise error rate of the whole comparison.
"""
import numpy as np

OUTPUTS = ("sheep", "wolves", "grass", "sheep_energy", "wolves_energy",
           "grass_countdown")
MEASURES = ("max", "argmax", "min", "argmin", "ss_mean", "ss_std")


def series(rows, cells):
    """(iters+1, 6) float64 outputs from (iters+1, 6) stats rows
    (sheep, wolves, grass, sheep_en, wolves_en, grass_en)."""
    r = np.asarray(rows, dtype=np.float64)
    out = np.empty_like(r)
    out[:, 0:3] = r[:, 0:3]
    with np.errstate(invalid="ignore", divide="ignore"):
        out[:, 3] = np.where(r[:, 0] > 0, r[:, 3] / np.maximum(r[:, 0], 1), 0.0)
        out[:, 4] = np.where(r[:, 1] > 0, r[:, 4] / np.maximum(r[:, 1], 1), 0.0)
    out[:, 5] = r[:, 5] / float(cells)
    return out


def focal_measures(rows, cells, ss_from):
    """(6 outputs, 6 measures) focal measures of one run."""
    x = series(rows, cells)
    ss = x[ss_from + 1:]
    fm = np.empty((6, 6))
    fm[:, 0] = x.max(axis=0)
    fm[:, 1] = x.argmax(axis=0)
    fm[:, 2] = x.min(axis=0)
    fm[:, 3] = x.argmin(axis=0)
    fm[:, 4] = ss.mean(axis=0)
    fm[:, 5] = ss.std(axis=0, ddof=1)
    return fm


def compare_samples(a, b):
    """p-value and test name for two 1-D samples."""
    from scipy import stats
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if np.ptp(a) == 0 and np.ptp(b) == 0:
        return (1.0 if a[0] == b[0] else 0.0), "constant"
    normal = True
    for s in (a, b):
        if np.ptp(s) == 0 or stats.shapiro(s).pvalue <= 0.05:
            normal = False
    if normal:
        return float(stats.ttest_ind(a, b, equal_var=False).pvalue), "welch-t"
    return float(stats.mannwhitneyu(a, b, alternative="two-sided").pvalue), "mann-whitney"


def holm(pvals):
    """Holm step-down adjusted p-values."""
    p = np.asarray(pvals, np.float64)
    order = np.argsort(p)
    m = len(p)
    adj = np.empty(m)
    run = 0.0
    for i, k in enumerate(order):
        run = max(run, min(1.0, (m - i) * p[k]))
        adj[k] = run
    return adj


def compare(fm_a, fm_b, alpha=0.05):
    """Compare two sets of replications, each an (n_reps, 6, 6) array of
    focal measures. Returns (passed, table) where table lists
    (output, measure, test, p, p_holm, mean_a, mean_b)."""
    fm_a = np.asarray(fm_a)
    fm_b = np.asarray(fm_b)
    rows = []
    for o in range(6):
        for m in range(6):
            p, test = compare_samples(fm_a[:, o, m], fm_b[:, o, m])
            rows.append([OUTPUTS[o], MEASURES[m], test, p,
                         float(fm_a[:, o, m].mean()), float(fm_b[:, o, m].mean())])
    adj = holm([r[3] for r in rows])
    table = [(r[0], r[1], r[2], r[3], float(adj[i]), r[4], r[5])
             for i, r in enumerate(rows)]
    passed = all(t[4] >= alpha for t in table)
    return passed, table


def raw_below(table, alpha=0.05):
    """Number of measures whose uncorrected p-value is below alpha. With 36
    measures and no difference about 36 x 0.05 = 1.8 are expected by chance
    (more spread than a binomial, because the measures are correlated)."""
    return sum(1 for t in table if t[3] < alpha)


def format_table(table):
    lines = ["%-16s %-7s %-13s %9s %9s %14s %14s" % (
        "output", "measure", "test", "p", "p_holm", "mean_a", "mean_b")]
    for t in table:
        lines.append("%-16s %-7s %-13s %9.4f %9.4f %14.4f %14.4f" % t)
    lines.append("uncorrected p < 0.05: %d of %d measures (about %.1f expected "
                 "by chance); smallest Holm-adjusted p: %.4f"
                 % (raw_below(table), len(table), 0.05 * len(table),
                    min(t[4] for t in table)))
    return "\n".join(lines)
