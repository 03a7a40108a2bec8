"""Named workloads of the Kobayashi step (synthetic, seeded).

Each builder returns plain Python/numpy data: parameters, grid size, the
initial nuclei as (cx, cy, r) disks and the step count.  Random choices use
splitmix64 (Steele, Lea & Flood 2014) so every run, on any machine, builds the
same workload.

  grid_300     300^2, one disk r=5, 2000 steps (the small parity case)
  grid_8192    8192^2, 64 non-overlapping disks r in {4..8}, 10,000 steps in
               CUDA-graph chunks of 100 (the throughput / roofline case)
  variants_2048  2048^2, one disk, j x delta x K x theta0 = 54 variants, 5,000 steps
  ensemble_512   512 instances, sides log-uniform in [64, 512], per-instance
               parameters, one disk r in {3..6}, 3,000 steps
  adjoint_512  512^2, 4,000 steps, target at delta=.04, K=1.8, theta0=.5,
               gradient at delta=.02, K=1.6, theta0=.2, T0 ~ N(0, 0.01^2)
"""
import math

import numpy as np

MASK64 = (1 << 64) - 1

BASE = dict(dx=0.03, dy=0.03, dt=1e-4, tau=3e-4, eps_bar=0.01, mu=1.0, K=1.6, delta=0.02, aniso=6.0, alpha=0.9,
            gamma=10.0, teq=1.0, theta0=0.2)


class SplitMix64:
    def __init__(self, seed):
        self.s = seed & MASK64

    def next(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & MASK64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * ((self.next() >> 11) * 2.0 ** -53)

    def randint(self, lo, hi):
        """uniform integer in [lo, hi] inclusive"""
        return lo + self.next() % (hi - lo + 1)

    def normal(self):
        u1 = self.uniform()
        u2 = self.uniform()
        return math.sqrt(-2.0 * math.log(1.0 - u1)) * math.cos(2.0 * math.pi * u2)


def periodic_dist2(a, b, n):
    d = abs(a - b) % n
    return min(d, n - d)


def grid_300():
    return dict(name="grid_300", nx=300, ny=300, params=dict(BASE), disks=[(150, 150, 5)], steps=2000)


def grid_8192(seed=8192, n_disks=64, n=8192):
    """the 8192^2 throughput case; other n give the same recipe on an n^2 grid (profiling cases)"""
    rng = SplitMix64(seed)
    disks = []
    while len(disks) < n_disks:
        cx, cy, r = rng.randint(0, n - 1), rng.randint(0, n - 1), rng.randint(4, 8)
        ok = all(math.hypot(periodic_dist2(cx, x, n), periodic_dist2(cy, y, n)) > r + rr for x, y, rr in disks)
        if ok:
            disks.append((cx, cy, r))
    return dict(name="grid_%d" % n, nx=n, ny=n, params=dict(BASE), disks=disks, steps=10000, chunk=100)


def variants_2048(steps=5000):
    out = []
    for j in (4, 6):
        for delta in (0.01, 0.02, 0.05):
            for K in (1.2, 1.6, 2.0):
                for th0 in (0.0, 0.2, math.pi / 4):
                    p = dict(BASE, aniso=float(j), delta=delta, K=K, theta0=th0)
                    out.append(dict(name="v_j%d_d%g_K%g_t%.4f" % (j, delta, K, th0), nx=2048, ny=2048, params=p,
                                    disks=[(1024, 1024, 5)], steps=steps))
    return out


def ensemble_512(seed=512, count=512, steps=3000):
    rng = SplitMix64(seed)
    inst = []
    for _ in range(count):
        side = int(round(math.exp(rng.uniform(math.log(64), math.log(512)))))
        p = dict(BASE, delta=rng.uniform(0.01, 0.06), aniso=float(4 if rng.next() & 1 else 6),
                 K=rng.uniform(1.2, 2.0), theta0=rng.uniform(0.0, math.pi / 2), tau=rng.uniform(2e-4, 4e-4))
        r = rng.randint(3, 6)
        inst.append(dict(nx=side, ny=side, params=p, disks=[(side // 2, side // 2, r)]))
    return dict(name="ensemble_512", instances=inst, steps=steps)


def adjoint_512(seed=4000, n=512, steps=4000):
    rng = SplitMix64(seed)
    t0 = np.array([0.01 * rng.normal() for _ in range(n * n)]).reshape(n, n)
    return dict(name="adjoint_512", nx=n, ny=n, steps=steps, checkpoint_every=64,
                target_params=dict(BASE, delta=0.04, K=1.8, theta0=0.5),
                params=dict(BASE, delta=0.02, K=1.6, theta0=0.2), disks=[(n // 2, n // 2, 5)], T0=t0)


def initial_fields(nx, ny, disks):
    """phi = 1 on the disks (periodic distance, di^2 + dj^2 <= r^2), T = theta = 0 --
    the numpy statement of kg_seed_disks, used to feed the CPU oracle."""
    phi = np.zeros((ny, nx))
    ii = np.arange(nx)[None, :]
    jj = np.arange(ny)[:, None]
    for cx, cy, r in disks:
        di = (ii - cx) % nx
        di = np.where(di > nx // 2, di - nx, di)
        dj = (jj - cy) % ny
        dj = np.where(dj > ny // 2, dj - ny, dj)
        phi[(di * di + dj * dj) <= r * r] = 1.0
    return phi, np.zeros((ny, nx)), np.zeros((ny, nx))
