"""The algorithm of the beam kernels' running sums (fsibe_2d_gb300/csrc/running_sum.cuh),
restated in Python and checked on the CPU against the serial FP64 loop, bit for bit.

integrate_position.f90:14-44 sums the beam's increments node by node in FP64.  Within one
binade the sequential FP64 sum is an integer sum on the binade's grid 2^g: s_(k+1) =
(m + RN(a_k / 2^g)) 2^g with ties to the even m + RN, exact while 2^52 < |m + RN| < 2^53.  The
GPU takes 32 steps at a time per warp (a scan of parity maps for the ties, a scan of the
increments), up to the first step that leaves the binade, which is an FP64 addition.  This
restatement follows the same steps one lane at a time; the GPU code is checked the same way by
test_gpu_running_sums.py."""
import math
import random
import struct

T52, T53, FRAC = 1 << 52, 1 << 53, (1 << 52) - 1


def bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def from_bits(b):
    return struct.unpack("<d", struct.pack("<Q", b & ((1 << 64) - 1)))[0]


def term_inc(a, g):
    """(a / 2^g rounded to the nearest integer, ok, tie); a tie returns its lower candidate."""
    ab = bits(a)
    ex = (ab >> 52) & 0x7FF
    ma = (ab & FRAC) | (T52 if ex else 0)
    sh = g - (ex - 1075 if ex else -1074)
    shc = min(max(sh, 1), 63)
    q, rem, half = ma >> shc, ma & ((1 << shc) - 1), 1 << (shc - 1)
    neg = ab >> 63
    ok = ma == 0 or (sh > 0 and ex != 0x7FF)
    tie = ma != 0 and rem == half
    if ma == 0:
        return 0, ok, tie
    if tie:
        return (-q - 1 if neg else q), ok, tie
    r = q + (1 if rem > half else 0)
    return (-r if neg else r), ok, tie


def running_sum(a, batch=32):
    """Exclusive prefix s_k of a in FP64 order, by integer batches; also the FP64 step count."""
    n = len(a)
    out = [0.0] * n
    cur, k, fp64_steps = 0.0, 0, 0
    while k < n:
        out[k] = cur                       # the FP64 step k
        cur = cur + a[k]
        k += 1
        fp64_steps += 1
        cb = bits(cur)
        ex = (cb >> 52) & 0x7FF
        if ex == 0 or ex == 0x7FF:
            continue
        negs = cb >> 63
        m = -((cb & FRAC) | T52) if negs else ((cb & FRAC) | T52)
        g, hi = ex - 1075, cb & ~FRAC
        blo, bhi = (-T53, -T52) if negs else (T52, T53)
        while k < n:
            incs, oks, ties = [], [], []
            for t in range(batch):
                inc, ok, tie = term_inc(a[k + t], g) if k + t < n else (0, False, False)
                incs.append(inc); oks.append(ok); ties.append(tie)
            par = m & 1                    # the parity maps: a tie makes the value even
            for t in range(batch):
                if ties[t]:
                    incs[t] += (par ^ incs[t]) & 1
                par = 0 if ties[t] else par ^ (incs[t] & 1)
            p, nok = 0, batch
            for t in range(batch):        # the scan, cut at the first step leaving the binade
                p += incs[t]
                if not (oks[t] and blo < m + p < bhi):
                    nok = t
                    break
            p = 0
            for t in range(nok):
                out[k + t] = from_bits(hi | (abs(m + p) & FRAC))
                p += incs[t]
            m += p
            if nok:
                cur = from_bits(hi | (abs(m) & FRAC))
            k += nok
            if nok < batch:
                break
    return out, fp64_steps


def serial(a):
    s, out = 0.0, []
    for x in a:
        out.append(s)
        s = s + x
    return out


def same(x, y):
    return all(bits(u) == bits(v) or (math.isnan(u) and math.isnan(v)) for u, v in zip(x, y))


def test_beam_like_rows():
    rng = random.Random(5)
    for n in (1, 7, 256, 1024):
        for seed in range(12):
            ds = 1.0 / n
            th = [0.1 * math.sin(3 * i / n + seed) + rng.uniform(-1e-3, 1e-3) for i in range(n)]
            td = [rng.uniform(-1, 1) * 1e-2 * math.cos(5 * i / n) for i in range(n)]
            for row in ([math.cos(t) * ds for t in th], [math.sin(t) * ds for t in th],
                        [-(d * math.sin(t) * ds) for t, d in zip(th, td)], [d * math.cos(t) * ds for t, d in zip(th, td)]):
                got, _ = running_sum(row)
                assert same(got, serial(row)), (n, seed)


def test_straight_beam_ties_stay_integer_steps():
    # a straight beam: every term is ds, a tie on the grid of every other binade
    n = 256
    row = [1.0 / (n - 1)] * n
    got, fp64 = running_sum(row)
    assert same(got, serial(row))
    assert fp64 <= 12, fp64  # one FP64 step a binade, not one a tie


def test_hard_rows():
    rng = random.Random(3)
    rows = [
        [1.0] + [2.0 ** -53] * 300 + [3 * 2.0 ** -53] * 300,
        [0.5] + [(1 + 2 * rng.randrange(4)) * 2.0 ** -54 for _ in range(600)],
        [1.0] + [-(2.0 ** -54)] * 200 + [-(3 * 2.0 ** -55)] * 200 + [2.0 ** -53] * 100,
        [1.0, -1.0] * 295 + [1e-300] * 10,
        [5e-324] * 590 + [1e-310] * 10,
        [1e300] * 600,
        [rng.uniform(-1, 1) * 10 ** rng.uniform(-20, 2) for _ in range(1000)],
        [(-1) ** i * (1 + i * 1e-3) for i in range(600)],
        [0.0, -0.0] * 300,
        [2.0 ** -(i % 60) for i in range(600)],
        [1.0, float("inf"), 2.0, float("nan"), 1.0],
    ]
    for row in rows:
        got, _ = running_sum(row)
        assert same(got, serial(row))
