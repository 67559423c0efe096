"""The CPU cluster-pair list builder (oracle/nblist_oracle.c), which the GPU list is
checked against bit for bit, is itself complete: on random boxes (uniform sites, a
non-cubic box, the column widths and cluster heights the autotuner tries, and the small-box
all-pairs form), every ordered site pair within the list radius under the minimum image
lies in exactly one entry of the list, in the entry's own periodic image, and no entry is
repeated."""
import numpy as np
import pytest

from oracle.pyoracle import nblist


def minimum_image_pairs(w, L, r):
    """Ordered pairs (i, j), i != j, with |w_i - w_j| < r under the minimum image, and the
    image of j that realizes it (w_i - (w_j + img L))."""
    d = w[:, None, :] - w[None, :, :]
    img = np.rint(d / L)
    d = d - img * L
    d2 = (d * d).sum(-1)
    np.fill_diagonal(d2, np.inf)
    i, j = np.nonzero(d2 < r * r)
    return i, j, img[i, j].astype(int), np.sqrt(d2[i, j])


@pytest.mark.parametrize("seed", range(12))
def test_list_covers_every_pair_once(seed):
    rng = np.random.default_rng(seed)
    L = rng.uniform(14.0, 26.0, size=3)
    n = int(rng.integers(300, 1500))
    x = rng.uniform(0, L[0], n) + L[0] * rng.integers(-1, 2, n)  # unwrapped positions
    y = rng.uniform(0, L[1], n)
    z = rng.uniform(0, L[2], n) - L[2] * rng.integers(0, 2, n)
    r = float(rng.uniform(3.0, 0.45 * L.min()))
    cw = min((8 * L.prod() / n) ** (1 / 3), 0.75 * r) * float(rng.choice([0.8, 1.0, 1.25]))
    ncx, ncy = max(1, int(L[0] // cw)), max(1, int(L[1] // cw))
    zcap = cw * float(rng.choice([0.75, 1.0, 1.5]))
    small = int(L[0] < 2 * r + 2 * L[0] / ncx or L[1] < 2 * r + 2 * L[1] / ncy or L[2] < 2 * r + 2 * max(cw, zcap))
    c = nblist(x, y, z, tuple(L), r, ncx, ncy, small, zcap)
    cl, pairs, img = c["clusters"], c["pairs"], c["shifts"]
    w = np.stack([x, y, z], 1)
    w = w - L * np.floor(w * (1.0 / L))
    # every site in exactly one cluster
    members = cl[cl >= 0]
    assert np.array_equal(np.sort(members), np.arange(n))
    # no entry twice
    keys = {(int(a), int(b), *map(int, s)) for (a, b), s in zip(pairs, img)}
    assert len(keys) == len(pairs)
    cluster_of = np.empty(n, int)
    for k, row in enumerate(cl):
        cluster_of[row[row >= 0]] = k
    i, j, im, dist = minimum_image_pairs(w, L, r)
    clear = np.abs(dist - r) > 1e-9  # pairs at the radius itself may go either way
    for a, b, s in zip(i[clear], j[clear], im[clear]):
        if small:
            assert (cluster_of[a], cluster_of[b], 0, 0, 0) in keys
        else:
            assert (cluster_of[a], cluster_of[b], *s) in keys, (a, b, s)
