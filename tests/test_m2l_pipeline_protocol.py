"""The barrier protocol of the persistent tcgen05 M2L pipeline (k_m2l_tc5 in
aboria_gb300/csrc/fmm.cu), restated as a model and run under random
interleavings of its producer warp, its MMA-issuing thread, its four
epilogue warps and the asynchronous completions (bulk copies, cp.async
groups, MMA commits), for every ring configuration the kernel is compiled
with (read from fmm.cu).

The model follows the kernel.  Blocks are numbered g = 0, 1, ... across the
CTA's tiles (nkb blocks per tile); the K operand (A) and the gathered W rows
(B) have rings of SA and SB stages.  Per block ga the producer first issues
the gathers of the blocks up to ga + D (each waits for `emptyB` of block
gb - SB and is one cp.async group), then waits until at most gb - ga - 1
groups are pending and arrives on `fullB` of block ga, then waits for
`emptyA` of block ga - SA and issues block ga's bulk copy (completing
`fullA`).  The MMA thread, per tile it, waits for `accempty[it % 2]` phase
(it - 2) / 2 (it >= 2), then per block c waits for `fullA` (parity (c / SA)
& 1) and `fullB` (parity (c / SB) & 1) and commits to `emptyA` and
`emptyB`, after the tile to `accfull[it % 2]`, after all tiles to
`mmadone`.  Each epilogue warp waits for `accfull[it % 2]` phase it / 2 and
arrives on `accempty[it % 2]`, which completes a phase with its fourth
arrival.

Checked: no deadlock; every parity wait waits for the phase it means (a
barrier is never two phases ahead of its waiter, which would make
try_wait.parity spin until its bound); each barrier's phases complete in
order; no epilogue warp arrives on a phase of `accempty` before the previous
one has completed; `mmadone` completes once, after everything.
"""
import random
import re
from pathlib import Path

import pytest

FMM = Path(__file__).resolve().parent.parent / "aboria_gb300" / "csrc" / "fmm.cu"


def _ternary(expr, nrb):
    """Evaluate a C++ constexpr chain `c ? a : b` over NRB."""
    expr = expr.strip()
    while expr.startswith("(") and expr.endswith(")"):
        expr = expr[1:-1].strip()
    depth = 0
    for q, ch in enumerate(expr):
        depth += ch == "("
        depth -= ch == ")"
        if ch == "?" and depth == 0:
            break
    else:
        return int(expr.rstrip("u"))
    nest, depth = 0, 0
    for k in range(q + 1, len(expr)):
        ch = expr[k]
        depth += ch == "("
        depth -= ch == ")"
        if depth == 0 and ch == "?":
            nest += 1
        elif depth == 0 and ch == ":":
            if nest == 0:
                break
            nest -= 1
    cond = expr[:q].replace("NRB", str(nrb))
    assert re.fullmatch(r"[\d\s=<>!]+", cond), cond
    return _ternary(expr[q + 1:k], nrb) if eval(cond) else _ternary(expr[k + 1:], nrb)


def ring_configs():
    src = FMM.read_text()
    body = src[src.index("template <int NRB> struct T5Cfg {"):]
    sa_expr = re.search(r"static constexpr int SA = ([^;]+);", body).group(1)
    sb_expr = re.search(r"static constexpr int SB = ([^;]+);", body).group(1)
    d_expr = re.search(r"static constexpr int D = ([^;]+);", body).group(1)
    out = {}
    for nrb in (1, 2, 3, 4):
        sa, sb = _ternary(sa_expr, nrb), _ternary(sb_expr, nrb)
        d = eval(d_expr.replace("SB", str(sb)).replace("SA", str(sa)))
        out[nrb] = (sa, sb, d)
    return out


def run(nkb, SA, SB, D, seed, tiles=3):
    rnd = random.Random(seed)
    done = {}  # barrier -> completed phases
    arrivals = {}  # count-4 barrier -> arrivals in its pending phase

    def c(b):
        return done.get(b, 0)

    def complete(b, phase):
        assert c(b) == phase, ("phase order", b, phase, c(b))
        done[b] = phase + 1

    def arrive4(b, phase):
        assert c(b) == phase, ("arrival for a later phase", b, phase, c(b))
        arrivals[b] = arrivals.get(b, 0) + 1
        if arrivals[b] == 4:
            arrivals[b] = 0
            complete(b, phase)

    def ready(b, phase):  # try_wait.parity(phase & 1), checked against aliasing
        assert c(b) <= phase + 1, ("barrier two phases ahead of its waiter", b, phase)
        return (c(b) & 1) != (phase & 1)

    total = nkb * tiles
    bulk, groups, mma = [], [], []
    gdone, ga, gb, cc = 0, 0, 0, 0
    pstate = "gathers"
    mt, mp, mstate = 0, 0, "acq"
    etile = [0, 0, 0, 0]  # per epilogue warp: the next tile it drains
    for _ in range(400000):
        acts = [a for a, on in (("A", bulk), ("G", gdone < len(groups)), ("M", mma),
                                ("P", pstate != "end"), ("C", mstate != "end")) if on]
        acts += [("E", w) for w in range(4) if etile[w] < tiles]
        if not acts:
            break
        a = rnd.choice(acts)
        if a == "A":
            q = bulk.pop(rnd.randrange(len(bulk)))
            complete(("fullA", q % SA), q // SA)
        elif a == "G":
            gdone += 1  # cp.async groups complete in issue order
        elif a == "M":
            q = mma.pop(0)  # MMA commits complete in issue order
            if q[0] == "mmadone":
                complete("mmadone", 0)
            elif q[0] == "accfull":
                complete(("accfull", q[1] % 2), q[1] // 2)
            elif q[0] == "emptyA":
                complete(("emptyA", q[1] % SA), q[1] // SA)
            else:
                complete(("emptyB", q[1] % SB), q[1] // SB)
        elif a == "P":
            if pstate == "gathers":
                if ga == total:
                    pstate = "end"
                    continue
                if gb < total and gb <= ga + D:
                    if gb >= SB and not ready(("emptyB", gb % SB), (gb - SB) // SB):
                        continue
                    groups.append(gb)
                    gb += 1
                    continue
                pstate = "signal"
            if pstate == "signal":
                if len(groups) - gdone > gb - ga - 1:
                    continue
                complete(("fullB", ga % SB), ga // SB)
                pstate = "bulk"
            if pstate == "bulk":
                if ga >= SA and not ready(("emptyA", ga % SA), (ga - SA) // SA):
                    continue
                bulk.append(ga)
                ga += 1
                pstate = "gathers"
        elif a == "C":
            if mstate == "acq":
                if mt == tiles:
                    mma.append(("mmadone",))
                    mstate = "end"
                    continue
                if mt >= 2 and not ready(("accempty", mt % 2), (mt - 2) // 2):
                    continue
                mstate = "blocks"
                mp = 0
            if mstate == "blocks":
                if mp == nkb:
                    mma.append(("accfull", mt))
                    mt += 1
                    mstate = "acq"
                    continue
                if ready(("fullA", cc % SA), cc // SA) and ready(("fullB", cc % SB), cc // SB):
                    mma.append(("emptyA", cc))
                    mma.append(("emptyB", cc))
                    cc += 1
                    mp += 1
        else:
            w = a[1]
            it = etile[w]
            if ready(("accfull", it % 2), it // 2):
                arrive4(("accempty", it % 2), it // 2)
                etile[w] += 1
    else:
        raise AssertionError("deadlock")
    if not all(e == tiles for e in etile) or mstate != "end" or pstate != "end":
        raise AssertionError("deadlock")
    assert c("mmadone") == 1 and cc == total and ga == total and gb == total
    assert c(("accfull", 0)) + c(("accfull", 1)) == tiles


def test_ring_configurations_are_read():
    cfg = ring_configs()
    assert set(cfg) == {1, 2, 3, 4}
    for SA, SB, D in cfg.values():
        assert SA >= 2 and 1 <= D < SB


@pytest.mark.parametrize("nrb", [1, 2, 3, 4])
def test_protocol_has_no_deadlock_or_phase_aliasing(nrb):
    SA, SB, D = ring_configs()[nrb]
    # block counts: the short cases around the ring depths and the orders'
    # own ceil(n^3 / 16) (orders 5..8: 8, 14, 22, 32); 1 to 4 tiles per CTA
    for nkb in list(range(1, 2 * SB + 3)) + [8, 14, 22, 32]:
        for tiles in (1, 2, 3, 4):
            for seed in range(4):
                run(nkb, SA, SB, D, seed, tiles)


def test_model_detects_gathers_ahead_by_the_ring_depth():
    """The check has teeth: with D = SB the producer waits for the MMAs of a
    block whose gathers it has not yet signalled."""
    with pytest.raises(AssertionError, match="deadlock"):
        run(8, 3, 4, 4, 0)
