"""The barrier protocol of the tcgen05 M2L pipeline (k_m2l_tc5 in
aboria_gb300/csrc/fmm.cu), restated as a model and run under random
interleavings of its producer warp, its MMA-issuing thread and the
asynchronous completions (bulk copies, cp.async groups, MMA commits), for
every ring configuration the kernel is compiled with (read from fmm.cu).

The model follows the kernel: the producer waits for `empty` of block p - S,
arrives on `fullA` (the bulk copy completes it later), issues block p's
gathers as one cp.async group and, once at most LAG groups are pending,
arrives on `fullB` for block p - LAG (the rest after its loop); the MMA
thread waits for `fullA` and `fullB` of block c with parity (c / S) & 1 and
commits to `empty`, then to `accb`.

Checked: no deadlock; every parity wait waits for the phase it means (a
barrier is never two phases ahead of its waiter, which would make
try_wait.parity spin until its bound); each barrier's phases complete in
block order; the epilogue's barrier completes once.
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
    s_expr = re.search(r"static constexpr int S = ([^;]+);", body).group(1)
    lag_expr = re.search(r"static constexpr int LAG = ([^;]+);", body).group(1)
    return {nrb: (_ternary(s_expr, nrb), _ternary(lag_expr, nrb)) for nrb in (1, 2, 3, 4)}


def run(nkb, S, LAG, seed):
    rnd = random.Random(seed)
    done = {}  # barrier -> completed phases

    def c(b):
        return done.get(b, 0)

    def complete(b, phase):
        assert c(b) == phase, ("phase order", b, phase, c(b))
        done[b] = phase + 1

    def ready(b, phase):  # try_wait.parity(phase & 1), checked against aliasing
        assert c(b) <= phase + 1, ("barrier two phases ahead of its waiter", b, phase)
        return (c(b) & 1) != (phase & 1)

    bulk, groups, mma = [], [], []
    gdone, p, cc = 0, 0, 0
    pstate, cstate = "issue", "loop"
    for _ in range(200000):
        acts = [a for a, on in (("A", bulk), ("G", gdone < len(groups)), ("M", mma),
                                ("P", pstate != "end"), ("C", cstate != "end")) if on]
        if not acts:
            break
        a = rnd.choice(acts)
        if a == "A":
            q = bulk.pop(rnd.randrange(len(bulk)))
            complete(("fullA", q % S), q // S)
        elif a == "G":
            gdone += 1  # cp.async groups complete in issue order
        elif a == "M":
            q = mma.pop(0)  # MMAs complete in issue order
            if q == "accb":
                complete("accb", 0)
            else:
                complete(("empty", q % S), q // S)
        elif a == "P":
            if pstate == "issue":
                if p == nkb:
                    pstate = "tail"
                    continue
                if p >= S and not ready(("empty", p % S), (p - S) // S):
                    continue
                bulk.append(p)
                groups.append(p)
                pstate = "lag" if p >= LAG else "next"
            if pstate == "lag":
                if len(groups) - gdone > LAG:
                    continue
                complete(("fullB", (p - LAG) % S), (p - LAG) // S)
                pstate = "next"
            if pstate == "next":
                p += 1
                pstate = "issue"
            elif pstate == "tail":
                if gdone < len(groups):
                    continue
                for q in range(max(p - LAG, 0), p):
                    complete(("fullB", q % S), q // S)
                pstate = "end"
        else:
            if cc == nkb:
                mma.append("accb")
                cstate = "end"
                continue
            st, f = cc % S, cc // S
            if ready(("fullA", st), f) and ready(("fullB", st), f):
                mma.append(cc)
                cc += 1
    else:
        raise AssertionError("deadlock")
    assert c("accb") == 1 and cc == nkb and p == nkb


def test_ring_configurations_are_read():
    cfg = ring_configs()
    assert set(cfg) == {1, 2, 3, 4}
    for S, LAG in cfg.values():
        assert 1 <= LAG < S


@pytest.mark.parametrize("nrb", [1, 2, 3, 4])
def test_protocol_has_no_deadlock_or_phase_aliasing(nrb):
    S, LAG = ring_configs()[nrb]
    # block counts: the short cases around the ring depth and the orders'
    # own ceil(n^3 / 8) (orders 5..8: 16, 27, 43, 64)
    for nkb in list(range(1, 2 * S + 3)) + [16, 27, 43, 64]:
        for seed in range(12):
            run(nkb, S, LAG, seed)


def test_model_detects_a_lag_at_the_ring_depth():
    """The check has teeth: with LAG = S the producer waits for MMAs of a
    block whose operands it has not yet signalled."""
    with pytest.raises(AssertionError, match="deadlock"):
        run(8, 3, 3, 0)
