"""The thread decomposition of k_lr_stats (zenav1-svt_gb300/csrc/zf_lr.cu),
emulated on the CPU: CTAs of 256 / (3 win - 1) rows over the unit's rows
extended by win/2, one thread per (row, row offset dr) building the row sums
of D[y][x] * D[y+dr][x+dc] over every shifted column window from a running
prefix, one thread per (row, window row) for M. Checked against the direct
definition of compute_stats (svtav1-dsp/src/restoration.rs:567-632:
M[a] = sum y_a x, H[a][b] = sum y_a y_b, y the win x win window in
column-major order) on random data, win 5 and 7, odd unit sizes."""
import numpy as np
import pytest


def direct(Dfull, X, uw, uh, WIN, off):
    h = WIN//2; W2 = WIN*WIN
    H = np.zeros((W2,W2), np.int64); M = np.zeros(W2, np.int64)
    for i in range(uh):
        for j in range(uw):
            y = np.array([Dfull[off+i+r-h, off+j+c-h] for c in range(WIN) for r in range(WIN)], np.int64)
            H += np.outer(y, y); M += y * X[i, j]
    return np.triu(H), M
def emu(Dfull, X, uw, uh, WIN, off):
    HALF = WIN//2; W2 = WIN*WIN; NDR = 2*WIN-1; ROWS = 256//(NDR+WIN)
    H = np.zeros(W2*W2, np.int64); M = np.zeros(W2, np.int64)
    Dat = lambda y, x: int(Dfull[off+y, off+x])
    for y0 in range(-HALF, uh+HALF, ROWS):
        y1 = min(uh+HALF, y0+ROWS)
        xi0, xi1 = max(y0,0), min(y1,uh)
        nh = NDR*(y1-y0)
        for t in range(256):
            if t < nh:
                dr = t % NDR - (WIN-1); y = y0 + t//NDR
                if not (y+dr >= -HALF and y+dr < uh+HALF): continue
                dc0 = 1 if dr < 0 else 0
                pre = [0]*WIN; rs = [[0]*WIN for _ in range(WIN)]
                win = [0]*WIN
                for k in range(WIN-1): win[k+1] = Dat(y+dr, -HALF+k)
                for x in range(-HALF, uw+HALF):
                    for k in range(WIN-1): win[k] = win[k+1]
                    win[WIN-1] = Dat(y+dr, x+WIN-1)
                    edge = x < HALF+1 or x >= uw-HALF
                    if edge:
                        for dc in range(WIN):
                            for sc in range(-HALF, HALF+1):
                                if sc+HALF+dc > WIN-1: continue
                                if x == sc: rs[dc][sc+HALF] -= pre[dc]
                                if x == sc+uw: rs[dc][sc+HALF] += pre[dc]
                    a = Dat(y, x)
                    for dc in range(WIN): pre[dc] += a*win[dc]
                for dc in range(WIN):
                    if 2*HALF+dc <= WIN-1: rs[dc][2*HALF] += pre[dc]
                for dc in range(dc0, WIN):
                    for ca in range(WIN-dc):
                        v = rs[dc][ca]
                        if v == 0: continue
                        for ra in range(max(0,-dr), min(WIN, WIN-dr)):
                            sr = ra - HALF
                            if y < sr or y >= sr+uh: continue
                            ia = ca*WIN+ra; ib = (ca+dc)*WIN+ra+dr
                            H[ia*W2+ib] += v
            elif t < nh + WIN*(xi1-xi0):
                q = t - nh; ra = q % WIN; i = xi0 + q//WIN; yy = i + ra - HALF
                acc = [0]*WIN; win = [0]*WIN
                for k in range(WIN-1): win[k+1] = Dat(yy, -HALF+k)
                for j in range(uw):
                    for k in range(WIN-1): win[k] = win[k+1]
                    win[WIN-1] = Dat(yy, j+HALF)
                    for ca in range(WIN): acc[ca] += win[ca]*int(X[i, j])
                for ca in range(WIN): M[ca*WIN+ra] += acc[ca]
            # threads beyond: idle
        assert nh + WIN*(xi1-xi0) <= 256, (nh, xi1-xi0)
    Hm = H.reshape(W2, W2)
    return np.triu(Hm), M, Hm


@pytest.mark.parametrize("win", [5, 7])
@pytest.mark.parametrize("uw,uh", [(11, 9), (16, 23), (7, 30)])
def test_stats_decomposition_matches_direct(win, uw, uh):
    rng = np.random.default_rng(win * 1000 + uw * 31 + uh)
    off = 10
    dfull = rng.integers(-1023, 1024, (uh + 2 * off + 8, uw + 2 * off + 8))
    x = rng.integers(-1023, 1024, (uh, uw))
    hd, md = direct(dfull, x, uw, uh, win, off)
    he, me, hm = emu(dfull, x, uw, uh, win, off)
    assert (np.tril(hm, -1) == 0).all()  # only the upper triangle is written
    assert (hd == he).all() and (md == me).all()
