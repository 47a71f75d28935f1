"""CPU model of the block-per-pair team hand-off of the int32 passes
(sw_pass.cuh, TEAM > 1): warps take every TEAM-th column strip of one pair,
the last lane of a warp writes the strip's right edge row by row, 31 steps
behind its first lane, into the next warp's buffer, publishes
(strip << 16) | rows written after every chunk (row field 0xFFFF once the strip
is complete) and -(X + 2) when it leaves the pair with strip X not complete;
the first lane copies the edge rows of a chunk two chunks ahead, after waiting
for them.  The reverse pass shares its best hit, bounds each strip's rows by
it at set-up and stops a warp whose next strip's band starts below the rows
still to search.

Random interleavings of the warps check that the protocol never deadlocks,
that every edge row a warp copies is the one its strip needs (written by the
strip to its left, not an older or newer strip), and that the reverse pass
still finds the first hit."""
import random

import pytest

KCH = 8       # pipeline steps per chunk of a 32-lane group
LAG = 31      # the last lane's lag behind the first
DONE = 0xFFFF


class Pair:
    def __init__(self, rng, team, nstrips, nrows, reverse):
        self.team, self.nstrips, self.nrows, self.reverse = team, nstrips, nrows, reverse
        # reverse: each strip's band starts lower down; a strip's first hit (if
        # any) lies inside its band
        self.slope = rng.choice([0, 3, 17, 60])
        self.hit = {}
        if reverse:
            for s in range(nstrips):
                start = self.row0(s)
                if start <= nrows and rng.random() < 0.3:
                    self.hit[s] = rng.randint(start, nrows)

    def row0(self, s):
        return 1 + s * self.slope if self.reverse else 1


class Warp:
    def __init__(self, w, pair):
        self.w, self.pair = w, pair
        self.strip = w
        self.state = "setup" if w < pair.nstrips else "end"
        self.best = None

    def limit(self, best):
        return self.pair.nrows if best is None else min(self.pair.nrows, best[0] - 1)


def simulate(seed, team, nstrips, nrows, reverse):
    rng = random.Random(seed)
    pair = Pair(rng, team, nstrips, nrows, reverse)
    prog = [-1] * team                       # published progress per warp
    edge = [dict() for _ in range(team)]     # buffer of warp w: row -> (strip, row)
    shared = {"best": None}                  # reverse: (row, strip)
    warps = [Warp(w, pair) for w in range(team)]
    rows_of = {}                             # strip -> its row limit at set-up

    def wait_ok(wp, r0):
        """Lane 0 of warp wp may copy rows [r0, r0 + KCH) of strip - 1's edge."""
        if wp.strip == 0 or r0 > wp.rows:
            return "go"
        need = ((wp.strip - 1) << 16) | min(r0 + KCH - 1, wp.rows)
        v = prog[(wp.w - 1) % team]
        if v <= -2:
            return "abort" if wp.strip - 1 >= -v - 2 else "go"
        return "go" if v >= need else "wait"

    def copy(wp, r0):
        if wp.strip == 0 or r0 > wp.rows:
            return
        src = edge[wp.w]
        prod_rows = rows_of.get(wp.strip - 1)
        assert prod_rows is not None, ("edge of a strip that has not started", wp.strip, r0)
        for r in range(r0, min(r0 + KCH - 1, wp.rows) + 1):
            if r < wp.row0:
                continue
            got = src.get(r)
            if r <= prod_rows:
                assert got == (wp.strip - 1, r), ("stale or missing edge row", wp.strip, r, got)
            else:  # past the left strip's limit: an older strip's row at most
                assert got is None or got[0] < wp.strip - 1, ("edge row from a newer strip", wp.strip, r, got)

    def setup(wp):
        wp.rows = wp.limit(shared["best"]) if reverse else nrows
        rows_of[wp.strip] = wp.rows
        wp.row0 = pair.row0(wp.strip)
        wp.st = wp.row0 - 1
        wp.nsteps = wp.rows + LAG
        wp.pending = [wp.st + 1, wp.st + 1 + KCH]   # the two chunks fetched at set-up
        wp.found = None
        wp.state = "fetch"

    def step(wp):
        """One action of warp wp; False when it is blocked."""
        if wp.state == "setup":
            setup(wp)
            return True
        if wp.state == "fetch":      # lane 0 copying the pending chunks, in order
            while wp.pending:
                r0 = wp.pending[0]
                ok = wait_ok(wp, r0)
                if ok == "wait":
                    return False
                if ok == "abort":
                    wp.state = "leave"
                    return True
                copy(wp, r0)
                wp.pending.pop(0)
            wp.state = "run"
            return True
        if wp.state == "run":        # KCH pipeline steps
            for _ in range(KCH):
                if wp.st < wp.nsteps:
                    i = wp.st - LAG + 1              # the last lane's row
                    if wp.row0 <= i <= wp.rows and wp.strip + 1 < nstrips:
                        edge[(wp.w + 1) % team][i] = (wp.strip, i)
                    i0 = wp.st + 1                   # the first lane's row
                    if reverse and wp.found is None and pair.hit.get(wp.strip) == i0 and i0 <= wp.rows:
                        wp.found = (i0, wp.strip)
                wp.st += 1
            if wp.strip + 1 < nstrips:
                written = DONE if wp.st >= wp.nsteps else max(0, min(wp.st - LAG, wp.rows))
                prog[wp.w] = (wp.strip << 16) | written
            if wp.st < wp.nsteps:
                wp.pending = [wp.st + 1 + KCH]
                wp.state = "fetch"
            else:
                wp.state = "strip_end"
            return True
        if wp.state == "strip_end":
            if reverse and wp.found is not None:
                b = shared["best"]
                shared["best"] = wp.found if b is None or wp.found < b else b
            wp.strip += team
            more = wp.strip < nstrips
            if reverse and more:
                b = shared["best"]
                if b is not None and b[0] <= 1:
                    more = False
                if more:
                    more = pair.row0(wp.strip) <= wp.limit(b)
            wp.state = "setup" if more else "leave"
            return True
        if wp.state == "leave":
            prog[wp.w] = -(wp.strip + 2)
            wp.state = "end"
            return True
        return False

    active = list(warps)
    for w in warps:
        if w.state == "end":
            prog[w.w] = -(w.strip + 2)
    for _ in range(10_000_000):
        live = [w for w in active if w.state != "end"]
        if not live:
            break
        rng.shuffle(live)
        if not any(step(w) for w in live[:rng.randint(1, len(live))]) and not any(step(w) for w in live):
            raise AssertionError("deadlock: %s" % [(w.w, w.state, w.strip) for w in live])
    else:
        raise AssertionError("no end")
    if reverse:
        exp = min(((r, s) for s, r in pair.hit.items()), default=None)
        assert shared["best"] == exp, (shared["best"], exp, pair.hit, pair.slope)


@pytest.mark.parametrize("reverse", [False, True])
@pytest.mark.parametrize("nstrips", [1, 2, 3, 4, 5, 9, 17])
def test_team_hand_off(reverse, nstrips):
    for seed in range(40):
        nrows = random.Random(seed).choice([1, 7, 8, 9, 40, 150, 400])
        simulate(1000 * nstrips + seed, 4, nstrips, nrows, reverse)


@pytest.mark.parametrize("bug", [
    ("written = DONE if wp.st >= wp.nsteps else max(0, min(wp.st - LAG, wp.rows))",
     "written = DONE if wp.st >= wp.nsteps else max(0, min(wp.st, wp.rows))"),   # the last lane's lag ignored
    ('return "go" if v >= need else "wait"', 'return "go"'),                       # no wait at all
])
def test_team_model_catches_planted_bugs(bug):
    """The checks have teeth: each planted protocol bug makes some interleaving
    copy an edge row that its strip does not need."""
    src = open(__file__).read()
    assert bug[0] in src
    ns = {}
    exec(compile(src.replace(bug[0], bug[1]).replace("def test_", "def _t_"), "planted", "exec"), ns)
    caught = 0
    for seed in range(60):
        try:
            ns["simulate"](seed, 4, 9, 150, seed % 2 == 1)
        except AssertionError:
            caught += 1
    assert caught > 0
