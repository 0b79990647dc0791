"""The pair slots of a line draw binned as runs (lineRunInfo and the
walkers in srp_gb300/csrc/k_front.cu), checked on the CPU: for random lines,
including long ones, ones on the framebuffer's edges and ones cut by a
scissor rectangle, the runs each walker finds (maximal sequences of
consecutive DDA steps that pass the scissor test, land in the framebuffer
and stay in one 8x8 tile) never exceed the slots its bound gives, and the
walkers' bounds add up to at most the line's slots. The DDA is the
reference's (src/raster/line.c:34-77): fp32 accumulators stepped serially,
rounded half away from zero."""
import math

import numpy as np

TILE, SHORT, MAXRUN = 8, 48, 15


def setup(x0, y0, x1, y1):
    dx, dy = np.float32(x1) - np.float32(x0), np.float32(y1) - np.float32(y0)
    steps = max(int(math.ceil(max(abs(dx), abs(dy)))), 1)
    return np.float32(x0), np.float32(y0), np.float32(dx / np.float32(steps)), np.float32(dy / np.float32(steps)), steps


def walk(x0, inc, n):
    """Accumulator values of steps 0..n (serial fp32 adds)."""
    v = np.empty(n + 1, np.float32)
    v[0] = x0
    acc = np.float32(x0)
    for s in range(1, n + 1):
        acc = np.float32(acc + inc)
        v[s] = acc
    return v


def rnd(v):
    return np.where(v >= 0, np.floor(v.astype(np.float64) + 0.5), -np.floor(-v.astype(np.float64) + 0.5)).astype(np.int64)


def far_pixel(v0, inc, n):
    e = float(v0) + n * float(inc)
    m = n * max(abs(float(v0)), abs(e)) * 2.0 ** -23 + 2.0 ** -10
    f = e + m if inc >= 0 else e - m
    r = math.floor(abs(f) + 0.5) * (1 if f >= 0 else -1)
    return int(max(min(r, 2e9), -2e9))


def tile_distance(ax, ay, bx, by):
    return abs(int(ax / TILE) - int(bx / TILE)) + abs(int(ay / TILE) - int(by / TILE))


def runs(px, py, W, H, sc):
    """Runs of the steps (px[i], py[i]) as the walker forms them."""
    keys = []
    for x, y in zip(px, py):
        key = None
        if sc is None or (sc[0] <= x < sc[2] and sc[1] <= y < sc[3]):
            idx = y * W + x
            if 0 <= idx < W * H:
                key = (idx // W // TILE, idx % W // TILE)
        keys.append(key)
    n, prev, count = 0, None, 0
    for k in keys:
        if k != prev or count == MAXRUN:
            if prev is not None and count:
                n += 1
            prev, count = k, 0
        if k is not None:
            count += 1
    if prev is not None and count:
        n += 1
    return n


def check_line(x0, y0, x1, y1, W, H, sc):
    X0, Y0, xi, yi, steps = setup(x0, y0, x1, y1)
    total = steps + 1
    xs, ys = walk(X0, xi, total), walk(Y0, yi, total)      # steps 0..total (one past the last)
    px, py = rnd(xs), rnd(ys)
    ax, ay = int(px[0]), int(py[0])
    bx, by = far_pixel(X0, xi, total), far_pixel(Y0, yi, total)
    inside = 0 <= ax < W and 0 <= ay < H and 0 <= bx < W and 0 <= by < H
    walkers = 1 if total <= SHORT else 32
    slots = min(total, tile_distance(ax, ay, bx, by) + walkers) if inside else total
    if walkers == 1:
        assert runs(px[:total], py[:total], W, H, sc) <= slots
        return inside
    seg = (total + 31) // 32
    used = 0
    for lane in range(32):
        s0, s1 = min(lane * seg, total), min(lane * seg + seg, total)
        mine = s1 - s0
        if inside and mine:
            nx, ny = (int(px[s1]), int(py[s1])) if lane < 31 else (bx, by)
            mine = min(mine, tile_distance(int(px[s0]), int(py[s0]), nx, ny) + 1)
        assert runs(px[s0:s1], py[s0:s1], W, H, sc) <= mine
        used += mine
    assert used <= slots
    return inside


def test_line_run_slots_bound_the_runs():
    rng = np.random.default_rng(7)
    W, H = 301, 203
    inside = 0
    for i in range(600):
        kind = i % 4
        if kind == 0:      # long, across the framebuffer
            x0, y0, x1, y1 = rng.uniform(0, W), rng.uniform(0, H), rng.uniform(0, W), rng.uniform(0, H)
        elif kind == 1:    # short
            x0, y0 = rng.uniform(0, W), rng.uniform(0, H)
            x1, y1 = x0 + rng.uniform(-20, 20), y0 + rng.uniform(-20, 20)
        elif kind == 2:    # ending on the right or bottom edge (the pixel index wraps a row there)
            x0, y0 = rng.uniform(0, W), rng.uniform(0, H)
            x1, y1 = (W, rng.uniform(0, H)) if rng.uniform() < 0.5 else (rng.uniform(0, W), H)
        else:              # nearly axis-aligned, many steps in one tile row or column
            x0, y0 = rng.uniform(0, W), rng.uniform(0, H)
            x1, y1 = (x0 + rng.uniform(-200, 200), y0 + rng.uniform(-1, 1)) if rng.uniform() < 0.5 else \
                     (x0 + rng.uniform(-1, 1), y0 + rng.uniform(-150, 150))
            x1, y1 = min(max(x1, 0), W), min(max(y1, 0), H)
        sc = None if i % 3 == 0 else (int(rng.integers(0, 60)), int(rng.integers(0, 40)),
                                      int(rng.integers(150, W + 40)), int(rng.integers(100, H + 30)))
        inside += check_line(x0, y0, x1, y1, W, H, sc)
    assert inside > 300   # most lines take the tile bound, not the step-per-slot fallback


def test_runs_in_one_tile_are_short():
    # a tile holds at most 10 consecutive steps of one line, well under the
    # 15 fragments a run may carry: the major-axis increment is at least 8/9
    # for lines of 8 pixels and more, and shorter lines have at most 9 steps
    rng = np.random.default_rng(3)
    longest = 0
    for _ in range(400):
        x0, y0 = rng.uniform(0, 100), rng.uniform(0, 100)
        x1, y1 = x0 + rng.uniform(-60, 60), y0 + rng.uniform(-60, 60)
        X0, Y0, xi, yi, steps = setup(x0, y0, x1, y1)
        px, py = rnd(walk(X0, xi, steps)), rnd(walk(Y0, yi, steps))
        run = 1
        for s in range(1, steps + 1):
            same = px[s] // TILE == px[s - 1] // TILE and py[s] // TILE == py[s - 1] // TILE
            run = run + 1 if same else 1
            longest = max(longest, run)
    assert longest <= 10
