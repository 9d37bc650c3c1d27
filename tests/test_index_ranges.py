"""The hot-path kernels' index arithmetic replayed on the CPU for every N
(compute-sanitizer is closed on the GPU pool): every global access stays
inside its buffer and every element of each output is written exactly once,
so no two threads race on a store.  Mirrors csrc/ocean_kernels.cu:
inter_index, LineOut::pos, the row-pass stores, k_col_fft's row gather, tile
copies and column-map stores, k_col_out's staged loads and output stores, and
the adjoint's column-pass loads and stores and row-pass dh0 updates
(csrc/ocean_adjoint.cu)."""
import numpy as np
import pytest

# LineFor / ColLineFor decompositions (R1, R2, R3) of csrc/fft_line.cuh and ocean_kernels.cu
LINE_FOR = {32: (8, 4, 1), 64: (8, 8, 1), 128: (16, 8, 1), 256: (16, 16, 1), 512: (16, 16, 2),
            1024: (16, 16, 4), 2048: (16, 16, 8)}
COL_LINE_FOR = {**LINE_FOR, 1024: (32, 32, 1), 2048: (32, 8, 8)}
SIZES = sorted(LINE_FOR)


def line(N, R):
    R1, R2, R3 = R[:3]
    R4 = R[3] if len(R) > 3 else 1
    G, E = N // R1, R1
    RL = R4 if R4 > 1 else (R3 if R3 > 1 else R2)
    NS = N // RL
    t = np.arange(G)[:, None]
    e = np.arange(E)[None, :]
    return G, E, R1, (e // RL) * G + (e % RL) * NS, t        # pos(0, e) and the thread index


def inter_rows(N):
    return N // 2 + 1


def inter_len(N):
    return 3 * inter_rows(N) * N


def inter_index(N, f, x, y):
    return ((f * (N // 2) + (x >> 1)) * inter_rows(N) + y) * 2 + (x & 1)


# the 8-point-first row lines of the warp-specialised row pass (RowLine<N, 2>)
ROW_LINE_V2 = {512: (8, 8, 8), 1024: (8, 8, 4, 4), 2048: (8, 8, 8, 4)}
ROW_CASES = [(N, LINE_FOR[N]) for N in SIZES] + sorted(ROW_LINE_V2.items()) + [(1024, (32, 32, 1))]


@pytest.mark.parametrize("N,R", ROW_CASES)
def test_row_pass_stores_cover_the_intermediate_once(N, R):
    G, E, R1, pos, t = line(N, R)
    H = inter_rows(N)
    x = t + pos                                                  # (G, E) output positions of a line
    assert np.array_equal(np.sort(x.ravel()), np.arange(N))
    assert np.all(pos % 2 == 0)
    hits = np.zeros(inter_len(N), np.int64)
    for f in range(3):
        for yp in range(H):
            idx = inter_index(N, f, t, yp) + (pos >> 1) * (2 * H)     # the kernels' store address
            assert np.array_equal(idx, inter_index(N, f, x, yp))
            np.add.at(hits, idx.ravel(), 1)
    assert np.all(hits == 1)


@pytest.mark.parametrize("N", SIZES)
def test_col_fft_gather_rows(N):
    """Input r of thread t is row y = t + r*G: read from row ys <= N/2,
    conjugated exactly when y > N/2 (the Hermitian half)."""
    G, E, R1, _, t = line(N, COL_LINE_FOR[N])
    r = np.arange(E)[None, :]
    y = t + r * G
    assert np.array_equal(np.sort(y.ravel()), np.arange(N))
    ys = np.where(r < R1 // 2, t + r * G, np.where(r == R1 // 2, N // 2 - t, N - t - r * G))
    cj = (r > R1 // 2) | ((r == R1 // 2) & (t != 0))
    assert np.array_equal(ys, np.where(y <= N // 2, y, N - y))
    assert np.array_equal(cj, y > N // 2)
    assert ys.min() >= 0 and ys.max() <= N // 2


@pytest.mark.parametrize("N", SIZES)
def test_col_fft_tile_copies_and_map_stores(N):
    G, E, R1, pos, t = line(N, COL_LINE_FOR[N])
    H = inter_rows(N)
    pairs = 1 if G >= 32 else 32 // G                             # ColCfg::PAIRS
    ctas = (N // 2) // pairs
    # three 1-D bulk copies per CTA: field f, pairs pair0 .. pair0+PAIRS-1, rows 0..N/2
    hits = np.zeros(inter_len(N), np.int64)
    for b in range(ctas):
        for f in range(3):
            s = inter_index(N, f, 2 * b * pairs, 0)
            hits[s:s + pairs * H * 2] += 1
    assert np.all(hits == 1)
    # column maps [3][N (x)][N (y)]: line f of pair (x0, x0+1) writes y = t + pos for both columns
    maps = np.zeros(3 * N * N, np.int64)
    for b in range(ctas):
        for pl in range(pairs):
            x0 = 2 * (b * pairs + pl)
            for f in range(3):
                o = (f * N + x0) * N + t + pos
                np.add.at(maps, o.ravel(), 1)
                np.add.at(maps, (o + N).ravel(), 1)
    assert np.all(maps == 1)


@pytest.mark.parametrize("N", SIZES)
def test_col_out_loads_and_stores(N):
    T, W, TH = 32, 34, 256                                       # kOutT, kOutW, kOutTh
    rows = T * T // TH
    ncol = 3 * W
    tid = np.arange(TH)
    out = np.zeros(N * N, np.int64)
    for bx in range(N // T):
        for by in range(N // T):
            x0, y0 = bx * T, by * T
            i = np.arange(ncol * 8)
            c = i >> 3
            f, xx = c // W, c % W
            ld = (f * N + ((x0 - 1 + xx) & (N - 1))) * N + y0 + 4 * (i & 7)
            assert ld.min() >= 0 and ld.max() + 3 < 3 * N * N and np.all(ld % 4 == 0)
            i = np.arange(2 * ncol)
            c = i >> 1
            f, xx = c // W, c % W
            yy = np.where(i & 1, (y0 + T) & (N - 1), (y0 - 1) & (N - 1))
            ld = (f * N + ((x0 - 1 + xx) & (N - 1))) * N + yy
            assert ld.min() >= 0 and ld.max() < 3 * N * N
            xs = tid % T + 1
            yb = (tid // T) * rows
            for k in range(rows):
                o = (y0 + yb + k) * N + x0 + xs - 1
                np.add.at(out, o, 1)
    assert np.all(out == 1)


@pytest.mark.parametrize("N", SIZES)
def test_adjoint_column_pass_loads_and_stores(N):
    """k_adj_col_pass (csrc/ocean_adjoint.cu): C columns per CTA, gy + i*gx
    lines per column and gz lines per column pair. Loads stay in the frame;
    every (field, ky <= N/2, x) of the frame's adjoint slab [3][H][N] is
    written once; the float4 Dz stores are 16-byte aligned."""
    G, E, R1, _, _ = line(N, LINE_FOR[N])
    C = 4 if N >= 2048 else 8
    WL, ZL = C, C // 2
    H = inter_rows(N)
    hits = np.zeros(3 * H * N, np.int64)
    for bx in range(N // C):
        x0 = bx * C
        u = np.arange(WL * G)                                     # gy + i*gx lines
        lane, t = u % WL, u // WL
        y = t[:, None] + np.arange(E)[None, :] * (N // R1)
        x = x0 + lane
        assert y.max() < N and x.max() < N
        u = np.arange(ZL * G)                                     # gz pair lines, float2 loads
        lane, t = u % ZL, u // ZL
        x = x0 + 2 * lane
        assert x.max() + 1 < N and np.all(x % 2 == 0)
        ky = np.arange(H)
        for c in range(WL):
            for f in (0, 1):
                np.add.at(hits, (f * H + ky) * N + x0 + c, 1)
        for p in range(ZL):
            o = (2 * H + ky) * N + x0 + 2 * p                     # float2 units
            assert np.all(o % 2 == 0)                             # 16-byte aligned float4 store
            np.add.at(hits, o, 1)
            np.add.at(hits, o + 1, 1)
    assert np.all(hits == 1)


@pytest.mark.parametrize("N", SIZES)
def test_adjoint_row_pass_accumulators_and_dh0(N):
    """k_adj_row_pass: within a frame each shared accumulator (pair, side,
    mx) has one writer. Across the CTAs, dh0 gets exactly one
    read-modify-write per (y, x): rows 0 and N/2 are their own mirrors and
    skip side 1."""
    G = N // LINE_FOR[N][0]
    pairs = 1 if G >= 32 else 32 // G
    H = inter_rows(N)
    dh0 = np.zeros(N * N, np.int64)
    for b in range((H + pairs - 1) // pairs):
        acc = np.zeros(2 * pairs * N, np.int64)
        for pl in range(pairs):
            yp = b * pairs + pl
            if yp >= H:
                continue
            yq = (N - yp) & (N - 1)
            kx = np.arange(N)
            np.add.at(acc, (pl * 2 + 0) * N + kx, 1)
            if yq != yp:
                np.add.at(acc, (pl * 2 + 1) * N + ((N - kx) & (N - 1)), 1)
            for side in (0, 1):
                y = yq if side else yp
                if side and y == yp:
                    continue
                np.add.at(dh0, y * N + kx, 1)
        assert acc.max() <= 1
    assert np.all(dh0 == 1)


@pytest.mark.parametrize("N", [512, 1024])
def test_col_fused_mirror_shuffles(N):
    """k_col_fused loads rows 0..N/2 only; register r > R1/2 of lane t (row
    N - t - r*G, the conjugate of a loaded row) comes from register R1-1-r of
    lane (32 - t) & 31, lane 0 from its own register R1 - r.  Both source
    registers are loaded ones, and they hold exactly the mirrored row."""
    G, E, R1, pos, t = line(N, COL_LINE_FOR[N])
    assert G == 32 and E == R1
    HR = R1 // 2
    lane = np.arange(32)
    loaded = {r: np.where(np.full(32, r < HR), lane + r * G, N // 2 - lane) for r in range(HR + 1)}
    for r in range(HR + 1):
        assert loaded[r].min() >= 0 and loaded[r].max() <= N // 2
    for r in range(HR + 1, R1):
        want = N - lane - r * G                                  # the row register r stands for, mirrored
        assert want.min() >= 1 and want.max() < N // 2
        src = (32 - lane) & 31
        got = loaded[R1 - 1 - r][src]
        got[0] = loaded[R1 - r][0]
        assert R1 - 1 - r < HR and R1 - r < HR
        assert np.array_equal(got, want)


@pytest.mark.parametrize("N,P", [(512, 2), (1024, 2), (512, 4), (1024, 4)])
def test_col_fused_loads_staging_and_stores(N, P):
    """k_col_fused<N, P>: every line load lies in the intermediate (16-byte
    pair loads aligned), each CTA's staged columns (two halo, 2P own) are
    written exactly once before the epilogue reads them, every staged read is
    in range and every output texel is written exactly once over the grid."""
    G, E, R1, pos, t = line(N, COL_LINE_FOR[N])
    assert G == 32
    LINES = 3 * (P + 1)
    COLS, CP, EROWS = 2 * P + 2, N + 16 // P, 32 * LINES // (2 * P)
    NPAD = N + N // R1
    assert 3 * COLS * CP <= 2 * LINES * NPAD                       # staging fits the exchange buffers
    r = np.arange(E)[None, :]
    ys = np.where(r < R1 // 2, t + r * G, np.where(r == R1 // 2, N // 2 - t, N - t - r * G))
    out_hits = np.zeros(N * N, np.int64)
    for b in range(N // (2 * P)):
        x0 = 2 * P * b
        stage = np.zeros(3 * COLS * CP, np.int64)
        for li in range(LINES):
            f, kind = li % 3, li // 3
            ca = x0 + 2 * kind if kind < P else (x0 - 1) & (N - 1)
            cb = ca + 1 if kind < P else (x0 + 2 * P) & (N - 1)
            for c in (ca, cb):
                idx = inter_index(N, f, c, ys)
                assert idx.min() >= 0 and idx.max() < inter_len(N)
            if kind < P:
                assert np.all(inter_index(N, f, ca, ys) % 2 == 0)         # float4 (pair) loads
            cA = 1 + 2 * kind if kind < P else 0
            cB = 2 + 2 * kind if kind < P else 2 * P + 1
            y = t + pos                                                   # LineOut positions
            for cc, col in ((cA, ca), (cB, cb)):
                assert col == (x0 - 1 + cc) & (N - 1)                     # staged column cc is x0 - 1 + cc
                np.add.at(stage, ((f * COLS + cc) * CP + y).ravel(), 1)
        used = np.zeros_like(stage, dtype=bool)
        for f in range(3):
            for cc in range(COLS):
                used[(f * COLS + cc) * CP:(f * COLS + cc) * CP + N] = True
        assert np.all(stage[used] == 1) and np.all(stage[~used] == 0)
        # epilogue, texel (x0 + c - 1, y) reading columns c-1..c+1, rows y-1..y+1.  4 pairs: thread
        # (c, q) walks rows [q*N/EBLK, (q+1)*N/EBLK) of staged column c; 2 pairs: thread tid
        # takes rows tid/2P + EROWS*k
        tid = np.arange(32 * LINES)
        c = tid % (2 * P) + 1
        if P == 4:
            EBLK = 32 * LINES // (2 * P)
            q = tid // (2 * P)
            ya, yb = q * N // EBLK, (q + 1) * N // EBLK
            assert ya.min() == 0 and yb.max() == N and np.all(yb > ya)
            steps = [(ya + k, ya + k < yb) for k in range((yb - ya).max())]
        else:
            steps = [(tid // (2 * P) + y0, tid // (2 * P) + y0 < N) for y0 in range(0, N, EROWS)]
        for y, keep in steps:
            y, cc = y[keep], c[keep]
            for dc in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    rd = (cc + dc) * CP + ((y + dy) & (N - 1))
                    assert rd.min() >= 0 and rd.max() < COLS * CP and np.all(used[rd])
            np.add.at(out_hits, y * N + x0 + cc - 1, 1)
    assert np.all(out_hits == 1)


@pytest.mark.parametrize("N,P,per_sm,threads,loop", [(1024, 4, 2, 224, False), (1024, 2, 2, 224, False),
                                                    (512, 2, 2, 224, False), (1024, 4, 4, 96, True),
                                                    (512, 2, 8, 96, True)])
def test_row_spectrum_prefetch(N, P, per_sm, threads, loop):
    """Single unit overlapping a fused column stage: CTAs 0..E-1 (E = SMs the
    column stage leaves free x row CTAs per SM) prefetch the spectrum rows of
    items E..N/2, each row pair exactly once, every prefetch a whole in-range
    row of the spectrum.  k_row_ws: one item per thread pair; k_row_pass
    (loop): thread pairs step on by E * threads/2 items."""
    sms, items = 152, N // 2 + 1
    grid = min(sms * per_sm, items)
    E = min(max(0, sms - N // (2 * P)) * per_sm, grid)
    seen = {}
    for b in range(E):
        for tid in range(threads):
            i = E + b + E * (tid >> 1)
            while i < items:
                row = (N - i) & (N - 1) if tid & 1 else i
                assert 0 <= row < N                               # a.spec + row*N, N float2
                seen[(i, tid & 1)] = seen.get((i, tid & 1), 0) + 1
                if not loop:
                    break
                i += E * (threads >> 1)
    assert all(v == 1 for v in seen.values())
    assert len(seen) == (2 * (items - E) if E > 0 else 0)       # no free SMs: no prefetch


@pytest.mark.parametrize("per_sm,expect_all_early", [(2, False), (3, True)])
def test_row_ws_second_jobs_go_to_early_ctas(per_sm, expect_all_early):
    """k_row_ws at N=1024 beside the 4-pair fused kernel: CTA b takes items b,
    b + grid, ...  The CTAs that start early are the first E = (152 - 128) *
    per_sm (the SMs the fused kernel leaves free).  At three CTAs per SM
    (row_variant 5) every CTA with a second job is an early one, so every
    late CTA has one job; at two (row_variant 3) most second jobs land on late
    CTAs."""
    N, sms, fused_ctas = 1024, 152, 1024 // 8
    items = N // 2 + 1
    grid = min(sms * per_sm, items)
    E = (sms - fused_ctas) * per_sm
    jobs = np.zeros(grid, np.int64)
    for item in range(items):
        jobs[item % grid] += 1
    assert jobs.sum() == items and jobs.max() <= 2
    two = np.nonzero(jobs == 2)[0]
    assert (two.size == 0 or two.max() < E) == expect_all_early
