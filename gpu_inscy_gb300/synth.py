"""Seeded synthetic subspace-cluster datasets for the five INSCY workloads.

The reference generates its synthetic data with a prebuilt binary
(`data/cluster_generator`, called from `python/inscy.py:239-257`) that is not
used here.  These generators follow the workload descriptions instead:
Gaussian clusters hidden in random axis-parallel subspaces (uniform in the
other dimensions), plus uniform noise, float32 in [0, 1], row-major [n, d],
rows shuffled.  Every dataset is a pure function of its seed.

Workloads (with the INSCY parameters each one is run with):

* ``small``   n=1,500, d=5: 4 clusters x 300 points, std 0.03, each in its own
  3-dim subspace; 300 noise points.  eps=0.05 F=1 num_obj=2 min_size=8 r=1
  cells=4.
* ``plain``   n=25,000, d=15: 10 clusters x 2,250, std 0.02, 4-6 dim
  subspaces; 2,500 noise points.  eps=0.03 F=1 num_obj=4 min_size=16 r=1
  cells=4.
* ``batch``   64 datasets, n log-uniform in [2,000, 50,000], d in [8, 20],
  3-8 clusters (std 0.02-0.05) in 3-6 dim subspaces, 5-20 % noise; the
  ``plain`` parameters.
* ``large_d`` n=100,000, d=25: 15 clusters with Zipf(1.2) sizes, std
  0.015-0.04, 3-8 dim subspaces, 15 % noise.  eps=0.02 num_obj=8 min_size=32
  cells=5.
* ``huge``    n=1,000,000, d=32: 20 clusters with Zipf(1.5) sizes, std
  0.01-0.05, 2-10 dim subspaces, 4 pairs of clusters sharing a subspace,
  30 % noise.  eps=0.015 num_obj=16 min_size=64 cells=6.
* ``real shapes``  stand-ins with the sizes of the reference's real-data
  runs (glass 214 x 9, vowel 990 x 10, pendigits 7,494 x 16, sky 7,300 x 17):
  Gaussian clusters (std 0.01-0.04) in 2-6 dim subspaces, 20 % noise, run with
  the reference's real-data parameters (cells=4, num_obj=8, F=1, r=1,
  min_size=0.05 n, eps=0.01, rectangular density).  The real datasets
  themselves are not used.
"""
import numpy as np

PARAMS = {
    "small": dict(neighborhood_size=0.05, F=1.0, num_obj=2, min_size=8, r=1.0, number_of_cells=4),
    "plain": dict(neighborhood_size=0.03, F=1.0, num_obj=4, min_size=16, r=1.0, number_of_cells=4),
    "batch": dict(neighborhood_size=0.03, F=1.0, num_obj=4, min_size=16, r=1.0, number_of_cells=4),
    "large_d": dict(neighborhood_size=0.02, F=1.0, num_obj=8, min_size=32, r=1.0, number_of_cells=5),
    "huge": dict(neighborhood_size=0.015, F=1.0, num_obj=16, min_size=64, r=1.0, number_of_cells=6),
}


def _zipf_sizes(rng, total, k, s):
    w = 1.0 / np.arange(1, k + 1, dtype=np.float64) ** s
    w = w[rng.permutation(k)]
    sizes = np.floor(total * w / w.sum()).astype(np.int64)
    sizes[np.argmax(sizes)] += total - sizes.sum()
    return sizes


def subspace_clusters(rng, n, d, sizes, stds, subspaces):
    """Place len(sizes) Gaussian clusters; the remaining rows are uniform noise."""
    X = rng.random((n, d), dtype=np.float64)
    row = 0
    for size, std, dims in zip(sizes, stds, subspaces):
        dims = np.asarray(dims)
        mu = rng.uniform(0.15, 0.85, size=len(dims))
        X[row:row + size, dims] = rng.normal(mu, std, size=(size, len(dims)))
        row += size
    np.clip(X, 0.0, 1.0, out=X)
    X = X[rng.permutation(n)]
    return np.ascontiguousarray(X.astype(np.float32))


def make_small(seed=0, n_clusters=4, per_cluster=300, noise=300, d=5, sub_dims=3, std=0.03):
    rng = np.random.default_rng(seed)
    n = n_clusters * per_cluster + noise
    subs = [np.sort(rng.choice(d, size=sub_dims, replace=False)) for _ in range(n_clusters)]
    return subspace_clusters(rng, n, d, [per_cluster] * n_clusters, [std] * n_clusters, subs)


def make_plain(seed=0, n=25_000, d=15, n_clusters=10, noise_frac=0.10, std=0.02, dims=(4, 6)):
    rng = np.random.default_rng(seed)
    n_noise = int(round(n * noise_frac))
    per = (n - n_noise) // n_clusters
    sizes = [per] * n_clusters
    subs = [np.sort(rng.choice(d, size=int(rng.integers(dims[0], dims[1] + 1)), replace=False))
            for _ in range(n_clusters)]
    return subspace_clusters(rng, n, d, sizes, [std] * n_clusters, subs)


def make_batch(seed=0, count=64, n_range=(2_000, 50_000), d_range=(8, 20)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]))))
        d = int(rng.integers(d_range[0], d_range[1] + 1))
        k = int(rng.integers(3, 9))
        noise = rng.uniform(0.05, 0.20)
        n_noise = int(round(n * noise))
        sizes = _zipf_sizes(rng, n - n_noise, k, 0.0)
        stds = rng.uniform(0.02, 0.05, size=k)
        subs = [np.sort(rng.choice(d, size=int(rng.integers(3, 7)), replace=False)) for _ in range(k)]
        out.append(subspace_clusters(rng, n, d, sizes, stds, subs))
    return out


def make_large_d(seed=0, n=100_000, d=25, n_clusters=15, noise_frac=0.15):
    rng = np.random.default_rng(seed)
    n_noise = int(round(n * noise_frac))
    sizes = _zipf_sizes(rng, n - n_noise, n_clusters, 1.2)
    stds = rng.uniform(0.015, 0.04, size=n_clusters)
    subs = [np.sort(rng.choice(d, size=int(rng.integers(3, 9)), replace=False)) for _ in range(n_clusters)]
    return subspace_clusters(rng, n, d, sizes, stds, subs)


def make_huge(seed=0, n=1_000_000, d=32, n_clusters=20, noise_frac=0.30):
    rng = np.random.default_rng(seed)
    n_noise = int(round(n * noise_frac))
    sizes = _zipf_sizes(rng, n - n_noise, n_clusters, 1.5)
    stds = rng.uniform(0.01, 0.05, size=n_clusters)
    subs = [np.sort(rng.choice(d, size=int(rng.integers(2, 11)), replace=False)) for _ in range(n_clusters)]
    for a in range(4):  # 4 pairs of clusters share a subspace
        subs[2 * a + 1] = subs[2 * a]
    return subspace_clusters(rng, n, d, sizes, stds, subs)


# name -> (n, d, clusters): the shapes of the reference's real-data runs
REAL_SHAPES = {"glass": (214, 9, 6), "vowel": (990, 10, 11), "pendigits": (7494, 16, 10), "sky": (7300, 17, 8)}


def real_params(n):
    """The reference's real-data run parameters for n points."""
    return dict(neighborhood_size=0.01, F=1.0, num_obj=8, min_size=int(0.05 * n), r=1.0, number_of_cells=4,
                rectangular=True)


def make_real_shape(name, seed=0):
    n, d, k = REAL_SHAPES[name]
    rng = np.random.default_rng(seed)
    n_noise = n // 5
    per = (n - n_noise) // k
    sizes = [per] * k
    sizes[-1] += n - n_noise - sum(sizes)
    stds = rng.uniform(0.01, 0.04, size=k)
    subs = [np.sort(rng.choice(d, size=int(rng.integers(2, min(d, 6) + 1)), replace=False)) for _ in range(k)]
    return subspace_clusters(rng, n, d, sizes, stds, subs)


def make_random(seed, n, d, n_clusters=2, std=0.04, sub_dims=None):
    """Small random instance for parity sweeps (n, d small)."""
    rng = np.random.default_rng(seed)
    n_noise = n // 4
    per = max(1, (n - n_noise) // max(1, n_clusters))
    sizes = [per] * n_clusters
    sizes[-1] += n - n_noise - sum(sizes)
    subs = []
    for _ in range(n_clusters):
        k = sub_dims if sub_dims is not None else int(rng.integers(1, d + 1))
        subs.append(np.sort(rng.choice(d, size=min(k, d), replace=False)))
    return subspace_clusters(rng, n, d, sizes, [std] * n_clusters, subs)


MAKERS = {"small": make_small, "plain": make_plain, "large_d": make_large_d, "huge": make_huge}
