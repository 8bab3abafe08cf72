"""The thread decomposition of k_lr_stats (zenav1-svt_gb300/csrc/zf_lr.cu),
emulated on the CPU: CTAs of 256 / (3 win) rows over the unit's rows
extended by win/2; one thread per (row, row offset dr) building the row sums
of d[y][x] * d[y+dr][x+dc] over every shifted column window from a running
prefix (head and tail steps at the window starts and ends, the middle in
plain steps or, for 8-bit rows with the 5-tap window, in four-column
groups on word boundaries); one thread per (unit row, window row) for M and
the window shift sums (a sliding column window); one thread per unit row
for the source sum and the three sse_region parts. The statistics are sums
of raw samples; the solve's average correction
    H = Hr - A (S_a + S_b) + n A^2,   M = Mr - A (S_a + sum s) + n A^2
is applied here as k_lr_solve does. Checked against the direct definition
of compute_stats (svtav1-dsp/src/restoration.rs:567-632: M[a] = sum y_a x,
H[a][b] = sum y_a y_b, y the win x win window of dgd - A in column-major
order, x = src - A, A = find_average) and sse_region on random data, win 5
and 7, narrow, odd and 16-multiple unit sizes."""
import numpy as np
import pytest


def direct(dfull, s, uw, uh, WIN, off):
    h = WIN // 2
    W2 = WIN * WIN
    A = int(dfull[off:off + uh, off:off + uw].sum()) // (uw * uh)
    H = np.zeros((W2, W2), np.int64)
    M = np.zeros(W2, np.int64)
    for i in range(uh):
        for j in range(uw):
            y = np.array([int(dfull[off + i + r - h, off + j + c - h]) - A for c in range(WIN) for r in range(WIN)],
                         np.int64)
            H += np.outer(y, y)
            M += y * (int(s[i, j]) - A)
    e2 = (s.astype(np.int64) - dfull[off:off + uh, off:off + uw].astype(np.int64)) ** 2
    dw, dh = uw % 16, uh % 16
    rgt = int(e2[:, uw - dw:].sum())
    bot = int(e2[uh - dh:, :uw - dw].sum())
    blk = int(e2[:uh - dh, :uw - dw].sum())
    return np.triu(H), M, (blk, rgt, bot)


def emu(dfull, s, uw, uh, WIN, off, packed):
    HALF = WIN // 2
    W2 = WIN * WIN
    NDR = 2 * WIN - 1
    ROWS = 256 // (NDR + WIN + 1)
    H = np.zeros(W2 * W2, np.int64)
    M = np.zeros(W2, np.int64)
    S = np.zeros(W2, np.int64)
    E = [0, 0, 0, 0]  # sum s, sse blocks, right, bottom
    Dat = lambda y, x: int(dfull[off + y, off + x])
    for y0 in range(-HALF, uh + HALF, ROWS):
        y1 = min(uh + HALF, y0 + ROWS)
        xi0, xi1 = max(y0, 0), min(y1, uh)
        nh = NDR * (y1 - y0)
        assert nh + (WIN + 1) * (xi1 - xi0) <= 256
        for t in range(nh):
            dr = t % NDR - (WIN - 1)
            y = y0 + t // NDR
            if not (-HALF <= y + dr < uh + HALF):
                continue
            dc0 = 1 if dr < 0 else 0
            pre = [0] * WIN
            rs = [[0] * WIN for _ in range(WIN)]
            win = [0] * WIN
            for k in range(WIN - 1):
                win[k + 1] = Dat(y + dr, -HALF + k)

            def step(x):
                for k in range(WIN - 1):
                    win[k] = win[k + 1]
                win[WIN - 1] = Dat(y + dr, x + WIN - 1)
                a = Dat(y, x)
                for dc in range(WIN):
                    pre[dc] += a * win[dc]

            xm0, xm1 = HALF + 1, max(HALF + 1, uw - HALF)
            if uw >= 16:
                for k in range(WIN):  # head: x = sc starts the windows of sc
                    for dc in range(WIN):
                        if k + dc <= WIN - 1:
                            rs[dc][k] -= pre[dc]
                    step(k - HALF)
                x = xm0
                if packed:
                    xs = HALF + 1 + ((4 - (2 * HALF + 1) % 4) & 3)
                    while x < xs:
                        step(x)
                        x += 1
                    if x + 4 <= xm1:
                        while x + 4 <= xm1:
                            assert (x + HALF) % 4 == 0  # word-aligned byte rows
                            for k in range(4):
                                a = Dat(y, x + k)
                                for dc in range(WIN):
                                    pre[dc] += a * Dat(y + dr, x + k + dc)
                            x += 4
                        for k in range(WIN - 1):
                            win[k + 1] = Dat(y + dr, x + k)
                else:
                    while x + WIN <= xm1:
                        for u in range(WIN):
                            step(x + u)
                        x += WIN
                while x < uw - HALF:
                    step(x)
                    x += 1
                for k in range(WIN):  # tail: x = sc + uw ends the windows of sc
                    for dc in range(WIN):
                        if k + dc <= WIN - 1:
                            rs[dc][k] += pre[dc]
                    if k < WIN - 1:
                        step(uw - HALF + k)
            else:
                for x in range(-HALF, uw + HALF):
                    for dc in range(WIN):
                        for sc in range(-HALF, HALF + 1):
                            if sc + HALF + dc > WIN - 1:
                                continue
                            if x == sc:
                                rs[dc][sc + HALF] -= pre[dc]
                            if x == sc + uw:
                                rs[dc][sc + HALF] += pre[dc]
                    step(x)
                for dc in range(WIN):
                    if 2 * HALF + dc <= WIN - 1:
                        rs[dc][2 * HALF] += pre[dc]
            for dc in range(dc0, WIN):
                for ca in range(WIN - dc):
                    v = rs[dc][ca]
                    for ra in range(max(0, -dr), min(WIN, WIN - dr)):
                        sr = ra - HALF
                        if y < sr or y >= sr + uh:
                            continue
                        ia, ib = ca * WIN + ra, (ca + dc) * WIN + ra + dr
                        H[ia * W2 + ib] += v
        for q in range(WIN * (xi1 - xi0)):
            ra = q % WIN
            i = xi0 + q // WIN
            yy = i + ra - HALF
            acc = [0] * WIN
            c0 = 0
            for j in range(uw):
                xv = int(s[i, j])
                for ca in range(WIN):
                    acc[ca] += Dat(yy, j + ca - HALF) * xv
                c0 += Dat(yy, j - HALF)
            for ca in range(WIN):
                M[ca * WIN + ra] += acc[ca]
            cw = c0
            S[ra] += cw
            for ca in range(1, WIN):  # the column windows slide
                cw = cw - Dat(yy, ca - 1 - HALF) + Dat(yy, ca - 1 - HALF + uw)
                S[ca * WIN + ra] += cw
        for i in range(xi0, xi1):  # sum s and the sse parts of unit row i
            jr = uw - uw % 16
            sx = e_in = e_rgt = 0
            j = 0
            if packed:  # four columns per step, then single columns
                while j + 4 <= uw:
                    for k in range(4):
                        xv = int(s[i, j + k])
                        e = xv - Dat(i, j + k)
                        sx += xv
                        if j >= jr:  # j and jr are multiples of 4
                            e_rgt += e * e
                        else:
                            e_in += e * e
                    j += 4
            while j < uw:
                xv = int(s[i, j])
                e = xv - Dat(i, j)
                sx += xv
                if j >= jr:
                    e_rgt += e * e
                else:
                    e_in += e * e
                j += 1
            E[0] += sx
            E[3 if i >= uh - uh % 16 else 1] += e_in
            E[2] += e_rgt
    # k_lr_solve's correction
    n = uw * uh
    ctr = HALF * WIN + HALF
    A = int(S[ctr]) // n
    Hm = H.reshape(W2, W2)
    Hc = np.zeros_like(Hm)
    for k in range(W2):
        for l in range(k, W2):
            Hc[k, l] = Hm[k, l] - A * (S[k] + S[l]) + n * A * A
    Mc = M - A * (S + E[0]) + n * A * A
    return Hc, Mc, Hm, (E[1], E[2], E[3])


@pytest.mark.parametrize("packed", [False, True])
@pytest.mark.parametrize("win", [5, 7])
@pytest.mark.parametrize("uw,uh", [(11, 9), (16, 23), (7, 30), (37, 18), (32, 16)])
def test_stats_decomposition_matches_direct(win, uw, uh, packed):
    if packed and win != 5:
        pytest.skip("the four-column path is the 5-tap window's")
    rng = np.random.default_rng(win * 1000 + uw * 31 + uh)
    off = 10
    hi = 256 if packed else 1024
    dfull = rng.integers(0, hi, (uh + 2 * off + 8, uw + 2 * off + 8))
    s = rng.integers(0, hi, (uh, uw))
    hd, md, ed = direct(dfull, s, uw, uh, win, off)
    he, me, hm, ee = emu(dfull, s, uw, uh, win, off, packed)
    assert (np.tril(hm, -1) == 0).all()  # only the upper triangle is written
    assert (hd == np.triu(he)).all() and (md == me).all()
    assert ed == ee
