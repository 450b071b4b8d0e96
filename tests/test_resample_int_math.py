"""The integer forms of the systematic resampler's draw description, as the
device walks it (resample_segments_kernel's build_segments and
resample_assign_kernel's count_below_fx in csrc/kernels.cu), restated here and
checked against the FP64 forms they replaced, on the CPU.

The reference's draws are U_{k+1} = (float)((double)U_k + 1.0/M)
(novel_resampling.h:59-63).  Inside one float binade [2^e, 2^(e+1)) they are
arithmetic: the double sum rounds 1/M to the binade's double ulp (Y units of
2^(e-52)), the float rounding turns that into R float ulps.  Both forms cut the
sequence into such segments plus single steps near each binade's top; they must
give the same segments, and the same count of draws below any sum c 2^-52."""
import math
import random
import struct

import numpy as np

M52 = (1 << 52) - 1


def f32(x):
    return float(np.float32(x))


def bits(d):
    return struct.unpack("<q", struct.pack("<d", d))[0]


def pow2(k):
    return math.ldexp(1.0, k)


def segments_fp64(M, u0, s_total, cap=1024):
    """The FP64 walk: rint / floor on doubles scaled by powers of two."""
    inv_m = 1.0 / M
    U, j, segs = float(u0), 0, []
    while U < s_total:
        if len(segs) == cap:
            return False, segs
        uf = f32(U)
        regular, cnt, delta = False, 0, 0.0
        if uf >= 1.17549435e-38:
            e = ((bits(U) >> 52) & 0x7FF) - 1023
            u, g, ginv = pow2(e - 23), pow2(e - 52), pow2(52 - e)
            y = float(np.rint(inv_m * ginv)) * g
            r = y * pow2(23 - e)
            if r - math.floor(r) == 0.5:
                return False, segs
            delta = float(np.rint(r)) * u
            if delta <= 0.0:
                return False, segs
            top = pow2(e + 1) - y
            if U < top:
                Ui, Di, Ti = int(U * ginv), int(delta * ginv), int(top * ginv)
                cnt = (Ti - Ui + Di - 1) // Di
                regular = cnt > 0
        if regular:
            segs.append((U, delta, j, cnt))
            j += cnt
            U = U + cnt * delta
        else:
            segs.append((U, 0.0, j, 1))
            j += 1
            nxt = f32(U + inv_m)
            if not nxt > U:
                return False, segs
            U = nxt
    return True, segs


def segments_int(M, u0, s_total, cap=1024):
    """The device's integer walk on the doubles' bits."""
    inv_m = 1.0 / M
    ib = bits(inv_m)
    Mi, Ei = (ib & M52) | (1 << 52), ((ib >> 52) & 0x7FF) - 1023
    U, j, segs = float(u0), 0, []
    s_bits = bits(s_total)
    while bits(U) < s_bits:
        if len(segs) == cap:
            return False, segs
        regular, cnt, D, e, Ui = False, 0, 0, 0, 0
        if bits(U) >= 0x3810000000000000:   # 2^-126
            ub = bits(U)
            e = ((ub >> 52) & 0x7FF) - 1023
            Ui = (ub & M52) | (1 << 52)
            sh = Ei - e
            big, Y = False, 0
            if sh >= 0:
                low = 0 if sh >= 29 else ((Mi & ((1 << (29 - sh)) - 1)) << sh)
                if sh >= 11:
                    big = True
                else:
                    Y = Mi << sh
                    big = Y >= (1 << 53)
            else:
                n = -sh
                if n < 64:
                    q, rem, half = Mi >> n, Mi & ((1 << n) - 1), 1 << (n - 1)
                    Y = q + (1 if (rem > half or (rem == half and q & 1)) else 0)
                low = Y & ((1 << 29) - 1)
            if low == 1 << 28:
                return False, segs
            if not big:
                R = (Y >> 29) + (1 if low > (1 << 28) else 0)
                if R == 0:
                    return False, segs
                D = R << 29
                T = (1 << 53) - Y
                if Ui < T:
                    cnt = ((T - Ui + D - 1) >> 29) // R
                    regular = cnt > 0
        if regular:
            segs.append((U, D * pow2(e - 52), j, cnt))
            j += cnt
            V = Ui + cnt * D
            U = pow2(e + 1) if V >= (1 << 53) else V * pow2(e - 52)
        else:
            segs.append((U, 0.0, j, 1))
            j += 1
            nxt = f32(U + inv_m)
            if not nxt > U:
                return False, segs
            U = nxt
    return True, segs


def count_fp64(segs, s):
    lo, hi = 0, len(segs)
    while lo < hi:
        mid = (lo + hi) // 2
        if segs[mid][0] < s:
            lo = mid + 1
        else:
            hi = mid
    if lo == 0:
        return 0
    u, d, j0, n = segs[lo - 1]
    if d == 0.0:
        return j0 + 1
    i = max(int((s - u) / d), 0)
    while i > 0 and u + (i - 1) * d >= s:
        i -= 1
    while i < n and u + i * d < s:
        i += 1
    return j0 + min(i, n)


def count_int(segs, c):
    """Draws below c 2^-52 (0 <= c < 2^53) with integer operations only."""
    sb = 0
    if c > 0:
        lz = 64 - c.bit_length()
        sb = ((63 - lz - 52 + 1023) << 52) | ((c << (lz - 11)) & M52)
    lo, hi = 0, len(segs)
    while lo < hi:
        mid = (lo + hi) // 2
        if bits(segs[mid][0]) < sb:
            lo = mid + 1
        else:
            hi = mid
    if lo == 0:
        return 0
    u, d, j0, n = segs[lo - 1]
    db = bits(d)
    if db == 0:
        return j0 + 1
    ub = bits(u)
    e, ed = ((ub >> 52) & 0x7FF) - 1023, ((db >> 52) & 0x7FF) - 1023
    A = ((ub & M52) | (1 << 52)) >> 29
    R = ((db & M52) | (1 << 52)) >> (e + 29 - ed)
    L = A + n * R
    t = -29 - e
    if t >= 0:
        S = L if (t >= 50 or (c >> (63 - t)) != 0) else (c << t)
        S = min(S, L)
    else:
        S = 1 if -t >= 63 else (c + (1 << -t) - 1) >> -t
    if S >= L:
        return j0 + n
    if S <= A:
        return j0
    return j0 + (S - A + R - 1) // R


def _cases(rng, n):
    out = []
    for k in range(n):
        M = rng.choice([1, 2, 3, 7, 1000, 65537, 100_000, 1_000_000, rng.randint(1, 2**24 - 1)])
        if k % 5 == 0:
            u0 = f32(rng.random() * 2.0 ** rng.randint(-140, -20))
        else:
            u0 = f32(rng.random() / M)
        s_total = f32(rng.uniform(0.5, 1.5)) if k % 7 else f32(2.0 ** rng.randint(-30, 12))
        out.append((M, u0, s_total))
    return out


def test_integer_segments_equal_fp64_walk():
    rng = random.Random(5)
    cases = _cases(rng, 400) + [(M, 0.0, 1.0) for M in (1, 2, 3, 100, 2**20)]
    for M, u0, s_total in cases:
        assert segments_int(M, u0, s_total) == segments_fp64(M, u0, s_total), (M, u0, s_total)


def test_integer_draw_counts_equal_fp64_search():
    rng = random.Random(9)
    checked = 0
    for M, u0, s_total in _cases(rng, 60):
        ok, segs = segments_int(M, u0, s_total)
        if not ok or not segs:
            continue
        for k in range(100):
            if k % 3 == 0:   # at and beside a draw
                u, d, j0, n = rng.choice(segs)
                v = u + rng.randint(0, max(0, n - 1)) * d
                c = int(round(v * 2.0**52)) + rng.randint(-2, 2)
            else:
                c = int(rng.random() * 2**52 * max(s_total, 1.0))
            c = max(0, min(c, 2**53 - 1))
            assert count_int(segs, c) == count_fp64(segs, math.ldexp(float(c), -52)), (M, u0, c)
            checked += 1
    assert checked > 3000
