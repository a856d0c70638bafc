"""Seeded synthetic netlists that stand in for the ISPD suites (absent here).

A netlist is what the placer's problem build (`src/database.py:11-100` of AutoPlace) produces from LEF + DEF:
cell sizes, pins as (cell, offset from the cell centre), pins grouped by net, the region, and the fixed objects.
Length unit: one site width; rows are `row_height` sites tall (site 0.2 um x row 2.0 um -> 10 sites).

Generator (one seed -> one netlist, bit for bit on every machine: numpy's PCG64 only):
  * cells: widths uniform integer 1..8 sites, one row tall;
  * locality: cell indices follow a Hilbert curve over the intended layout, so a net draws its pins from a window
    of +/- `window` cell indices around a random centre (no duplicate cell in a net);
  * degrees: 2 (60 %), 3 (20 %), uniform 4..10 (18 %), uniform 11..100 (2 %);
  * pin offsets uniform inside the cell;
  * square region at `util` of the free area; fixed macros (sides uniform 5..15 % of the region side, scaled to
    cover `macro_cover` of the region, no overlap, snapped to whole rows); a share of the nets ends on a macro pin
    (a fixed pin: cell index = num_mov, offset = absolute position).
"""
import math
from dataclasses import dataclass, field

import numpy as np

ROW_HEIGHT = 10.0


def areas(size):
    """[n, 2] sizes -> [n] float64 areas, the same values as size.prod(1) (one product per row), without numpy's slow
    reduction over a two-element axis."""
    a = np.asarray(size, np.float64)
    return a[:, 0] * a[:, 1]


@dataclass
class Netlist:
    name: str
    width: float
    height: float
    row_height: float
    size: np.ndarray            # [C, 2] float64, real cell sizes
    pin_cell: np.ndarray        # [P] int64, C = fixed pin
    pin_off: np.ndarray         # [P, 2] float64, offset from the cell centre (fixed pin: absolute position)
    pin_net: np.ndarray         # [P] int64, sorted
    num_nets: int
    macros: np.ndarray          # [M, 4] float64 (x0, y0, x1, y1)
    params: dict = field(default_factory=dict)

    @property
    def num_mov(self):
        return len(self.size)

    @property
    def num_pins(self):
        return len(self.pin_cell)

    @property
    def mov_area(self):
        key = (id(self.size), self.size.shape)          # (computed once per size array)
        if self.__dict__.get("_mov_area_key") != key:
            self.__dict__["_mov_area_key"] = key
            self.__dict__["_mov_area"] = float(areas(self.size).sum())
        return self.__dict__["_mov_area"]

    @property
    def cell_pins(self):
        return np.bincount(self.pin_cell, minlength=self.num_mov + 1)[:self.num_mov].astype(np.float64)

    def fixed_fraction(self, nbx, nby):
        """[nbx, nby] share of each bin under a macro (the rows cover the whole region here, and macros do not
        overlap), the quantity of `PlaceData.fixed_fraction` (`src/database.py:103-134`)."""
        bx, by = self.width / nbx, self.height / nby
        ex = np.arange(nbx + 1) * bx
        ey = np.arange(nby + 1) * by
        cover = np.zeros((nbx, nby))
        for x0, y0, x1, y1 in self.macros:
            ox = np.clip(np.minimum(ex[1:], x1) - np.maximum(ex[:-1], x0), 0, None)
            oy = np.clip(np.minimum(ey[1:], y1) - np.maximum(ey[:-1], y0), 0, None)
            cover += np.outer(ox, oy)
        return np.clip(cover / (bx * by), 0.0, 1.0)


PRESETS = {
    # name: cells, nets, window, macros, macro cover, target density, overflow grid, force grid (0 = rule), cluster
    # ratio (5: two levels, the reference's default, main.py:44)
    "c0": dict(cells=10_000, nets=10_500, window=200, macros=0, cover=0.0, target=1.0, num_bin=128, force_bin=0,
               cluster_ratio=5.0),
    "c1": dict(cells=200_000, nets=210_000, window=200, macros=20, cover=0.15, target=0.9, num_bin=0, force_bin=512,
               cluster_ratio=5.0),
    "c2": dict(cells=1_200_000, nets=1_250_000, window=2000, macros=40, cover=0.20, target=0.8, num_bin=512,
               force_bin=1024, cluster_ratio=5.0),
}


def _degrees(rng, n):
    u = rng.random(n)
    d = np.where(u < 0.6, 2, np.where(u < 0.8, 3, 0))
    mid = (u >= 0.8) & (u < 0.98)
    d[mid] = rng.integers(4, 11, int(mid.sum()))
    big = u >= 0.98
    d[big] = rng.integers(11, 101, int(big.sum()))
    return d.astype(np.int64)


def _net_cells(rng, deg, num_cells, window):
    """Distinct cells of every net from a window of 2 window + 1 indices. -> flat cell list grouped by net."""
    w = min(2 * window + 1, num_cells)
    lo = np.clip(rng.integers(0, num_cells, len(deg)) - window, 0, num_cells - w)
    out = [None] * len(deg)
    for d in np.unique(deg):
        idx = np.nonzero(deg == d)[0]
        if d <= 10:
            pick = rng.integers(0, w, (len(idx), d))
            for _ in range(64):                          # redraw the rows with a repeated cell
                s = np.sort(pick, 1)
                bad = np.nonzero((s[:, 1:] == s[:, :-1]).any(1))[0]
                if len(bad) == 0:
                    break
                pick[bad] = rng.integers(0, w, (len(bad), d))
            else:
                raise RuntimeError("could not draw distinct pins")
        else:
            pick = np.stack([rng.choice(w, d, replace=False) for _ in idx]) if len(idx) else np.zeros((0, d), int)
        cells = pick + lo[idx, None]
        for k, i in enumerate(idx):
            out[i] = cells[k]
    return np.concatenate(out) if out else np.zeros(0, np.int64)


def _place_macros(rng, count, cover, side, row_height):
    if count == 0 or cover <= 0:
        return np.zeros((0, 4))
    dims = rng.uniform(0.05, 0.15, (count, 2)) * side
    dims *= math.sqrt(cover * side * side / float(areas(dims).sum()))
    dims[:, 1] = np.maximum(np.round(dims[:, 1] / row_height), 1) * row_height
    dims[:, 0] = np.maximum(np.round(dims[:, 0]), 1)
    placed = []
    for w, h in dims:
        for _ in range(10_000):
            x0 = float(np.floor(rng.uniform(0, side - w)))
            y0 = float(np.floor(rng.uniform(0, side - h) / row_height) * row_height)
            r = (x0, y0, x0 + w, y0 + h)
            if all(r[2] <= q[0] or q[2] <= r[0] or r[3] <= q[1] or q[3] <= r[1] for q in placed):
                placed.append(r)
                break
        else:
            raise RuntimeError("could not place the macros without overlap")
    return np.array(placed, dtype=np.float64)


def make_netlist(cells, nets, window=200, macros=0, cover=0.0, util=0.7, fixed_pin_share=0.01, seed=0,
                 name=None, **_ignored):
    rng = np.random.default_rng(seed)
    size = np.stack([rng.integers(1, 9, cells).astype(np.float64), np.full(cells, ROW_HEIGHT)], 1)
    mov_area = float(areas(size).sum())
    region = mov_area / util / (1.0 - cover)
    side = math.ceil(math.sqrt(region) / ROW_HEIGHT) * ROW_HEIGHT
    mac = _place_macros(rng, macros, cover, side, ROW_HEIGHT)

    deg = np.minimum(_degrees(rng, nets), min(2 * window + 1, cells))   # a net fits in its window
    pin_cell = _net_cells(rng, deg, cells, window)
    pin_net = np.repeat(np.arange(nets, dtype=np.int64), deg)
    pin_off = (rng.random((len(pin_cell), 2)) - 0.5) * size[pin_cell]
    if len(mac) and fixed_pin_share > 0:              # the last pin of some nets is on a macro
        last = np.cumsum(deg) - 1
        sel = last[rng.random(nets) < fixed_pin_share]
        m = mac[rng.integers(0, len(mac), len(sel))]
        pin_cell[sel] = cells
        pin_off[sel, 0] = m[:, 0] + rng.random(len(sel)) * (m[:, 2] - m[:, 0])
        pin_off[sel, 1] = m[:, 1] + rng.random(len(sel)) * (m[:, 3] - m[:, 1])
    return Netlist(name or "synth_%d_s%d" % (cells, seed), float(side), float(side), ROW_HEIGHT, size,
                   pin_cell.astype(np.int64), pin_off, pin_net, int(nets), mac,
                   dict(cells=cells, nets=nets, window=window, macros=macros, cover=cover, util=util, seed=seed))


def preset(name, seed=0, **over):
    """Netlist of a preset (c0: 10k cells, c1: 200k cells + 20 macros, c2: 1.2M cells + 40 macros) and its run
    options: -> (netlist, options dict with target_density, num_bin, force_num_bin, cluster_ratio)."""
    p = dict(PRESETS[name])
    p.update(over)
    nl = make_netlist(seed=seed, name="%s_s%d" % (name, seed), **p)
    return nl, {"target_density": p["target"], "num_bin": p["num_bin"], "force_num_bin": p["force_bin"],
                "cluster_ratio": p["cluster_ratio"]}


def init_positions(nl, num_nodes, seed=0):
    """Cells in a small Gaussian cloud at the region centre, fillers uniform over the region (the start of
    `init_positions`, `src/initializer.py:40-47`), drawn with numpy -> float32 [num_nodes, 2]."""
    rng = np.random.default_rng(seed + 7_919)
    region = np.array([nl.width, nl.height], dtype=np.float32)
    cells = rng.standard_normal((nl.num_mov, 2)).astype(np.float32) * region * np.float32(0.001) + region * np.float32(0.5)
    fill = rng.random((num_nodes - nl.num_mov, 2)).astype(np.float32) * region
    return np.concatenate([cells, fill]).astype(np.float32)


def batch_instances(count=64, seed=0, lo=5_000, hi=150_000):
    """The batched workload (config 3): `count` seeded netlists with cell counts log-uniform in [lo, hi], nets 1.05 x
    cells, the config-0 degree mix and window, 0-10 macros (over 3-15 % of the region when there are any), one level
    each (cluster ratio 1), each with its own force grid by the grid rule (about one cell per free bin: 64 .. 512).
    -> list of (netlist, options dict)."""
    rng = np.random.default_rng(7_777 + seed)
    out = []
    for k in range(count):
        cells = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        macros = int(rng.integers(0, 11))
        cover = float(rng.uniform(0.03, 0.15)) if macros else 0.0
        nl = make_netlist(cells, int(round(cells * 1.05)), window=200, macros=macros, cover=cover,
                          seed=100_000 * (seed + 1) + k, name="c3_%d_%d" % (seed, k))
        out.append((nl, {"target_density": 1.0, "num_bin": 0, "force_num_bin": 0, "cluster_ratio": 1.0}))
    return out
