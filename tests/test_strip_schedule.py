"""CPU model of the bulk-copy (TMA) row schedule of the marching strip.

kg_strip (crystalgrowth_gb300/csrc/kg_device.cuh) stages the rows of phi and T
into two 8-slot shared-memory rings with cp.async.bulk, one row ahead of use,
and tracks every copy with one of 16 mbarriers (arrival count 1).  A wait on
an mbarrier names the parity of the phase it waits for, so a wrong ring
index or parity either passes before the copy has landed or waits on a phase
that never completes.  The GPU only reports the second kind, as a bounded-wait
time-out; the first kind silently reads stale rows, or lets the CTA exit with
a copy still in flight into shared memory that the next CTA then owns.

This test reads the slot and parity formulas out of the kernel source, replays
the strip's issue/wait/read order for every strip height 1..69 and 200 (and
for grids whose last strip is clipped), and checks:
  - every wait is for a row whose copy has been issued (no wait on nothing);
  - the awaited row's copy is the k-th arrival on its mbarrier with k of the
    parity the wait names, and the next arrival on that mbarrier has not been
    issued yet (otherwise the phase could run past the wait);
  - a ring slot is refilled only after the last read of the row it held;
  - every row read by stage 1 or stage 2 was waited for first;
  - at the strip's end, and at every possible failure exit, no copy is left
    in flight (on a failure exit, counting the extra bounded waits).
"""
import os
import re

import pytest

SRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "crystalgrowth_gb300", "csrc",
                   "kg_device.cuh")


def _lambda_expr(src, name):
    """the returned expression of `auto name = [&](int q) { return EXPR; };`"""
    m = re.search(r"auto\s+%s\s*=\s*\[&\]\(int q\)\s*\{\s*return\s+(.*?);\s*\};" % name, src)
    assert m, "kg_strip no longer defines %s as a one-line lambda; update this model" % name
    return m.group(1)


def _to_python(expr):
    e = expr.replace("(unsigned)", "").replace("1u", "1")
    m = re.fullmatch(r"&sm\.mbar\[(.*)\]", e)
    if m:
        e = m.group(1)
    assert re.fullmatch(r"[\sA-Za-z0-9_()+\-&>]*", e), "unexpected tokens in %r" % expr
    return e


@pytest.fixture(scope="module")
def formulas():
    src = open(SRC).read()
    out = {}
    for name in ("phi_bar", "phi_par", "t_bar", "t_par"):
        code = compile(_to_python(_lambda_expr(src, name)), name, "eval")
        out[name] = code
    # the issue-ahead distances and the loop bounds this model replays
    for stmt in ("issue_phi(j0 - 2);", "issue_phi(j0 - 1);", "issue_phi(j0);", "issue_t(j0 - 1);",
                 "wait_phi(j0 - 2);", "wait_phi(j0 - 1);", "for (int r = j0 - 1; r <= jend; r++)",
                 "if (r + 2 <= jend + 1)", "issue_phi(r + 2);", "if (r + 1 <= jend)", "issue_t(r + 1);",
                 "wait_phi(r + 1);", "wait_t(r);", "const int last_phi = min(r_fail + 2, jend + 1), last_t = min(r_fail + 1, jend);",
                 "for (int q = max(j0 - 2, last_phi - 7); q <= last_phi; q++)",
                 "for (int q = max(j0 - 1, last_t - 7); q <= last_t; q++)"):
        assert stmt in src, "kg_strip's schedule changed (%r not found); update this model" % stmt
    # the data slots of both rings
    assert "sm.phi[(q - base) & 7]" in src and "sm.t[(q - base) & 7]" in src
    return out


class Strip:
    """Replays one strip: thread 0's issues and the CTA's waits and shared-memory reads, in program order.

    Thread 0 issues the copies at the top of march iteration r, while the other threads may still be
    computing iteration r-1 (they have passed that iteration's row barrier, not yet the next one), so a
    refill issued at iteration r may only overwrite a row whose last read was in iteration r-2 or earlier."""

    def __init__(self, f, j0, bh, ny):
        self.f = f
        self.j0, self.jend, self.base = j0, min(j0 + bh, ny), j0 - 2
        self.arrivals = {}     # mbarrier -> [(ring, row)] in issue order
        self.issued = {}       # (ring, row) -> (mbarrier, arrival index)
        self.owner = {}        # (ring, slot) -> row held by the slot
        self.last_read = {}    # (ring, row) -> iteration of its latest read so far
        self.waited = set()    # (ring, row)
        self.errors = []
        self.it = None         # current march iteration (None: prologue)

    def ev(self, name, q):
        return eval(self.f[name], {}, {"q": q, "base": self.base, "j0": self.j0})

    def issue(self, ring, q):
        bar = self.ev("phi_bar" if ring == "phi" else "t_bar", q)
        slot = (q - self.base) & 7
        old = self.owner.get((ring, slot))
        if old is not None:
            if (ring, old) not in self.waited:
                self.errors.append("%s row %d refills slot %d before row %d was waited" % (ring, q, slot, old))
            lr = self.last_read.get((ring, old))
            if lr is not None and self.it is not None and lr > self.it - 2:
                self.errors.append("%s row %d refills slot %d at iteration %d; row %d was read at iteration %d"
                                   % (ring, q, slot, self.it, old, lr))
        k = len(self.arrivals.setdefault(bar, []))
        self.arrivals[bar].append((ring, q))
        self.issued[(ring, q)] = (bar, k)
        self.owner[(ring, slot)] = q

    def wait(self, ring, q):
        if (ring, q) not in self.issued:
            self.errors.append("wait on %s row %d, which was never issued" % (ring, q))
            return
        bar, k = self.issued[(ring, q)]
        par = self.ev("phi_par" if ring == "phi" else "t_par", q)
        if par != (k & 1):
            self.errors.append("%s row %d: arrival %d on mbarrier %d waited with parity %d" % (ring, q, k, bar, par))
        if len(self.arrivals[bar]) > k + 1:
            nxt = self.arrivals[bar][k + 1]
            self.errors.append("%s row %d: mbarrier %d already has the next arrival (%s row %d) before the wait"
                               % (ring, q, bar, nxt[0], nxt[1]))
        self.waited.add((ring, q))

    def read(self, ring, q):
        slot = (q - self.base) & 7
        if self.owner.get((ring, slot)) != q:
            self.errors.append("read of %s row %d from slot %d, which holds row %s"
                               % (ring, q, slot, self.owner.get((ring, slot))))
        elif (ring, q) not in self.waited:
            self.errors.append("read of %s row %d before its wait" % (ring, q))
        self.last_read[(ring, q)] = self.it

    def run(self, r_fail=None):
        """the march of kg_strip's bulk-copy path; r_fail: a row whose waits are made to give up"""
        j0, jend = self.j0, self.jend
        self.issue("phi", j0 - 2)
        self.issue("phi", j0 - 1)
        self.issue("phi", j0)
        self.issue("t", j0 - 1)
        self.wait("phi", j0 - 2)
        self.wait("phi", j0 - 1)
        failed_at = None
        for r in range(j0 - 1, jend + 1):
            self.it = r
            if r + 2 <= jend + 1:
                self.issue("phi", r + 2)
            if r + 1 <= jend:
                self.issue("t", r + 1)
            if r == r_fail:
                failed_at = r  # the waits of this row give up; every thread leaves at the row barrier
                break
            self.wait("phi", r + 1)
            self.wait("t", r)
            for q in (r - 1, r, r + 1):  # stage 1 at row r
                self.read("phi", q)
            s = r - 1  # stage 2 at row s, output rows j0 .. jend-1
            if j0 <= s < jend:
                for q in (s - 1, s, s + 1):
                    self.read("phi", q)
                    self.read("t", q)
        if failed_at is not None:
            last_phi, last_t = min(failed_at + 2, jend + 1), min(failed_at + 1, jend)
            for q in range(max(j0 - 2, last_phi - 7), last_phi + 1):
                self.wait("phi", q)
            for q in range(max(j0 - 1, last_t - 7), last_t + 1):
                self.wait("t", q)
        left = sorted(k for k in self.issued if k not in self.waited)
        if left:
            self.errors.append("copies in flight at exit: %s" % left)
        return self.errors


HEIGHTS = list(range(1, 70)) + [200]


@pytest.mark.parametrize("bh", HEIGHTS)
def test_schedule_full_strips(formulas, bh):
    for j0 in (0, bh, 3 * bh):
        errs = Strip(formulas, j0, bh, ny=j0 + bh + 5).run()
        assert not errs, errs[:5]


@pytest.mark.parametrize("bh", HEIGHTS)
def test_schedule_clipped_last_strip(formulas, bh):
    """ny cuts the strip short: jend = ny < j0 + bh"""
    for cut in sorted({1, 2, 3, max(1, bh // 2), max(1, bh - 1)}):
        if cut > bh:
            continue
        j0 = 2 * bh
        errs = Strip(formulas, j0, bh, ny=j0 + cut).run()
        assert not errs, (cut, errs[:5])


@pytest.mark.parametrize("bh", [1, 2, 3, 7, 8, 9, 15, 16, 17, 33, 64, 69, 200])
def test_schedule_failure_exits(formulas, bh):
    """a wait that gives up at any row: the extra bounded waits leave no copy in flight"""
    j0 = bh
    for r_fail in range(j0 - 1, j0 + bh + 1):
        errs = Strip(formulas, j0, bh, ny=j0 + bh + 3).run(r_fail=r_fail)
        assert not errs, (r_fail, errs[:5])


def test_model_catches_the_old_t_ring_numbering(formulas):
    """the T ring once numbered its arrivals from j0-2 like phi: the model must flag that"""
    bad = dict(formulas)
    bad["t_bar"] = compile("8 + ((q - base) & 7)", "t_bar", "eval")
    bad["t_par"] = compile("((q - base) >> 3) & 1", "t_par", "eval")
    errs = Strip(bad, 16, 16, ny=64).run()
    assert errs, "the model accepted a T ring whose first wait uses the wrong parity"
