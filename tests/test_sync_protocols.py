"""Host models of the synchronisation protocols of the persistent kernels,
checked exhaustively on small cases (the kernels themselves run in the GPU
tests):

* ``grid_barrier`` (csrc/tnc_persist.cuh): one atomic add per CTA, CTA 0 adds
  0x80000000 - (nblocks - 1) and the others 1; the top bit of the counter
  flips exactly when the last CTA of a barrier arrives, whatever the order.
* the step counters of ``jacobi_block_kernel`` (csrc/tnc_svd_rows.cu): a task
  of step g waits until both its half-blocks have completed g steps and
  publishes g + 1 after storing them; with CTAs interleaved at random (and
  fewer CTAs than tasks) every half-block sees its steps in order and the
  schedule never deadlocks.
"""
import random

M32 = 1 << 32


def test_grid_barrier_phase_bit():
    rng = random.Random(0)
    for n in (1, 2, 3, 8, 32, 64, 152, 304):
        count = 0
        for _ in range(8):
            order = list(range(n))
            rng.shuffle(order)
            base = count
            for idx, b in enumerate(order):
                add = (0x80000000 - (n - 1)) % M32 if b == 0 else 1
                old = count
                count = (count + add) % M32
                flipped = ((count ^ base) & 0x80000000) != 0
                last = (((old + add) % M32 ^ old) & 0x80000000) != 0
                assert flipped == (idx == n - 1)
                assert last == (idx == n - 1)
                assert ((old ^ base) & 0x80000000) == 0  # waiters saw the pre-flip phase


def _circle_pair(np_, r, i):
    mod = np_ - 1
    if i == 0:
        return r, mod
    return (r + i) % mod, (r - i + mod) % mod


def _run_schedule(nr, h, grid, sweeps, seed):
    rnd = random.Random(seed)
    nb = (nr + h - 1) // h
    nbp = nb + (nb & 1)
    ntask = nbp // 2
    ver = [0] * nb
    last = [-1] * nb

    def cta(b):
        for s in range(sweeps):
            g0 = s * nbp
            for hb in range(b, nb, grid):              # phase 0: ordered by the sweep barrier
                assert last[hb] == g0 - 1 and ver[hb] == g0
                last[hb] = g0
                yield "work"
                ver[hb] = g0 + 1
            for r in range(nbp - 1):
                g = g0 + 1 + r
                for t in range(b, ntask, grid):
                    P, Q = _circle_pair(nbp, r, t)
                    if P >= nb or Q >= nb:             # paired with the padding block
                        Pr = P if P < nb else Q
                        while ver[Pr] < g:
                            yield "wait"
                        assert last[Pr] == g - 1
                        last[Pr] = g
                        ver[Pr] = g + 1
                        continue
                    while ver[P] < g or ver[Q] < g:
                        yield "wait"
                    assert last[P] == g - 1 and last[Q] == g - 1
                    last[P] = last[Q] = g
                    yield "work"
                    ver[P] = ver[Q] = g + 1
            yield "barrier"

    ctas = [cta(b) for b in range(grid)]
    done = [False] * grid
    parked = set()
    idle = 0
    while not all(done):
        live = [b for b in range(grid) if not done[b] and b not in parked]
        if not live:
            parked.clear()                              # every live CTA reached the sweep barrier
            continue
        b = rnd.choice(live)
        try:
            ev = next(ctas[b])
        except StopIteration:
            done[b] = True
            continue
        if ev == "barrier":
            parked.add(b)
            if len(parked) == done.count(False):
                parked.clear()
        idle = idle + 1 if ev == "wait" else 0
        assert idle < 200000, "deadlock"
    assert ver == [sweeps * nbp] * nb


def test_jacobi_step_counters():
    for nr in (2, 3, 5, 16, 17, 31, 64, 100, 512):
        for h in (2, 4, 8, 16):
            nb = (nr + h - 1) // h
            ntask = (nb + (nb & 1)) // 2
            for grid in sorted({1, max(1, ntask // 3), max(1, ntask - 1), ntask}):
                _run_schedule(nr, h, grid, 2, seed=nr * 31 + h + grid)
