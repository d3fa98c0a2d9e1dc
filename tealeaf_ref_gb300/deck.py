"""TeaLeaf input decks: reader, writer and the seeded synthetic-problem generator.

The reader accepts the ``*tea ... *endtea`` block format of the reference
(parse.f90:143-247: case-folded, ``!``/``;`` start comments, ``=`` and ``,`` are
separators) and the keywords/defaults of read_input.f90:39-331.  The writer emits
a deck that the reference's reader accepts, so an identical input can be fed to a
Fortran build of the reference wherever one exists.

The seeded generator builds the synthetic problems used for parity and for
measurement (256^2 .. 8192^2 with random rectangles/circles).  Its random stream is
SplitMix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number generators",
OOPSLA 2014), mapped to doubles in [0,1) with the top 53 bits.
"""
from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

GEOMETRY_IDS = {"rectangle": 1, "circle": 2, "point": 3}
GEOMETRY_NAMES = {v: k for k, v in GEOMETRY_IDS.items()}

SOLVER_IDS = {"jacobi": 1, "cg": 2, "chebyshev": 3, "ppcg": 4}
CONDUCTIVITY = 1
RECIP_CONDUCTIVITY = 2
PREC_IDS = {"none": 1, "jac_diag": 2, "jac_block": 3}
PREC_NAMES = {v: k for k, v in PREC_IDS.items()}


def _f32(x: float) -> float:
    """Value of a Fortran default-REAL literal (single precision) widened to REAL(8)."""
    return float(np.float32(x))


@dataclass
class State:
    density: float = 0.0
    energy: float = 0.0
    geometry: int = 1  # 1 rectangle, 2 circle, 3 point
    xmin: float = 0.0
    xmax: float = 0.0
    ymin: float = 0.0
    ymax: float = 0.0
    radius: float = 0.0


@dataclass
class Deck:
    """Settings of one TeaLeaf run.  Defaults are read_input.f90:39-101."""

    states: List[State] = field(default_factory=list)
    x_cells: int = 10
    y_cells: int = 10
    xmin: float = 0.0
    ymin: float = 0.0
    xmax: float = 100.0
    ymax: float = 100.0
    initial_timestep: float = _f32(0.1)
    end_time: float = 10.0
    end_step: int = 640000  # g_ibig, data.f90:28
    summary_frequency: int = 10
    visit_frequency: int = 0
    max_iters: int = 1000
    eps: float = _f32(1.0e-10)
    solver: str = "jacobi"
    coefficient: int = CONDUCTIVITY
    preconditioner: str = "none"
    reflective_boundary: bool = False
    halo_depth: int = 1
    ch_cg_presteps: int = 25
    ch_cg_epslim: float = 1.0
    ppcg_inner_steps: int = -1
    check_result: bool = False
    test_problem: int = 0
    profiler_on: bool = False
    verbose_on: bool = False
    tiles_per_task: int = 1
    # read and kept for the record; a GPU chunk is one tile (read_input.f90:175-184, 221)
    sub_tiles_per_tile: int = 1
    tiles_per_problem: int = 0
    use_fortran_kernels: bool = True

    @property
    def solver_id(self) -> int:
        return SOLVER_IDS[self.solver]

    @property
    def precond_id(self) -> int:
        return PREC_IDS[self.preconditioner]

    @property
    def dx(self) -> float:
        # initialise_chunk.f90:34 (REAL() of the cell count is exact here)
        return (self.xmax - self.xmin) / float(np.float32(self.x_cells))

    @property
    def dy(self) -> float:
        return (self.ymax - self.ymin) / float(np.float32(self.y_cells))

    def effective_inner_steps(self) -> int:
        """tl_ppcg_inner_steps after the PPCG default of read_input.f90:324-327."""
        if self.ppcg_inner_steps == -1 and self.solver == "ppcg":
            cells = np.float32(self.x_cells * self.y_cells)
            return 4 * int(np.sqrt(np.sqrt(cells, dtype=np.float32), dtype=np.float32))
        return self.ppcg_inner_steps

    def state_arrays(self):
        """Per-state arrays (state 1 first) as passed to the chunk generator."""
        s = self.states
        return (
            np.array([x.density for x in s], dtype=np.float64),
            np.array([x.energy for x in s], dtype=np.float64),
            np.array([x.xmin for x in s], dtype=np.float64),
            np.array([x.xmax for x in s], dtype=np.float64),
            np.array([x.ymin for x in s], dtype=np.float64),
            np.array([x.ymax for x in s], dtype=np.float64),
            np.array([x.radius for x in s], dtype=np.float64),
            np.array([x.geometry for x in s], dtype=np.int32),
        )

    def replace(self, **kw) -> "Deck":
        d = dataclasses.replace(self, **kw)
        d.states = [dataclasses.replace(s) for s in self.states]
        return d


def _clean_lines(text: str):
    inside = False
    for raw in text.splitlines():
        line = "".join(ch if 32 <= ord(ch) <= 128 else " " for ch in raw).strip()
        for cmt in ("!", ";"):
            pos = line.find(cmt)
            if pos >= 0:
                line = line[:pos]
        line = line.strip().lower()
        if not line:
            continue
        if line.startswith("*"):
            word = line.split()[0]
            if word == "*tea":
                inside = True
            elif word == "*endtea":
                inside = False
            continue
        if inside:
            yield line.replace("=", " ").replace(",", " ").split()


def _rval(word: str) -> float:
    # parse_getrval: a number without a decimal point is read as if it had one
    return float(word)


def parse_deck(text: str) -> Deck:
    """Parse a ``*tea`` deck (read_input.f90:106-331)."""
    d = Deck()
    lines = list(_clean_lines(text))
    nstates = 0
    for words in lines:
        if words and words[0] == "state":
            nstates = max(nstates, int(words[1]))
    if nstates < 1:
        raise ValueError("read_input: No states defined.")
    d.states = [State() for _ in range(nstates)]
    defined = [False] * nstates
    for words in lines:
        it = iter(range(len(words)))
        i = 0
        while i < len(words):
            w = words[i]
            nxt = words[i + 1] if i + 1 < len(words) else None
            if w == "state":
                sid = int(nxt) - 1
                if defined[sid]:
                    raise ValueError("read_input: State defined twice.")
                defined[sid] = True
                st = d.states[sid]
                i += 2
                while i < len(words):
                    key = words[i]
                    val = words[i + 1] if i + 1 < len(words) else None
                    if key == "geometry":
                        st.geometry = GEOMETRY_IDS.get(val, st.geometry)
                    elif key in ("xmin", "xmax", "ymin", "ymax", "radius", "density", "energy"):
                        setattr(st, key, _rval(val))
                    else:
                        i += 1
                        continue
                    i += 2
                break
            consumed = 2
            if w == "initial_timestep":
                d.initial_timestep = _rval(nxt)
            elif w == "end_time":
                d.end_time = _rval(nxt)
            elif w == "end_step":
                d.end_step = int(nxt)
            elif w in ("xmin", "xmax", "ymin", "ymax"):
                setattr(d, w, _rval(nxt))
            elif w in ("x_cells", "y_cells", "visit_frequency", "summary_frequency", "tiles_per_task",
                       "sub_tiles_per_tile", "tiles_per_problem"):
                setattr(d, w, int(nxt))
            elif w == "tl_ch_cg_presteps":
                d.ch_cg_presteps = int(nxt)
            elif w == "tl_ppcg_inner_steps":
                d.ppcg_inner_steps = int(nxt)
            elif w == "tl_ch_cg_epslim":
                d.ch_cg_epslim = _rval(nxt)
            elif w == "tl_max_iters":
                d.max_iters = int(nxt)
            elif w == "tl_eps":
                d.eps = _rval(nxt)
            elif w == "halo_depth":
                d.halo_depth = int(nxt)
                if d.halo_depth < 1:
                    raise ValueError("read_input: Invalid halo exchange depth specified")
            elif w == "test_problem":
                d.test_problem = int(nxt)
            elif w == "tl_preconditioner_type":
                if nxt not in PREC_IDS:
                    raise ValueError("read_input: Invalid preconditioner type specified: %s" % nxt)
                d.preconditioner = nxt
            else:
                consumed = 1
                if w == "tl_check_result":
                    d.check_result = True
                elif w == "tl_use_jacobi":
                    d.solver = "jacobi"
                elif w == "tl_use_cg":
                    d.solver = "cg"
                elif w == "tl_use_ppcg":
                    d.solver = "ppcg"
                elif w == "tl_use_chebyshev":
                    d.solver = "chebyshev"
                elif w == "reflective_boundary":
                    d.reflective_boundary = True
                elif w == "profiler_on":
                    d.profiler_on = True
                elif w == "verbose_on":
                    d.verbose_on = True
                elif w == "use_fortran_kernels":
                    d.use_fortran_kernels = True
                elif w == "tl_coefficient_density":
                    d.coefficient = CONDUCTIVITY
                elif w == "tl_coefficient_inverse_density":
                    d.coefficient = RECIP_CONDUCTIVITY
            i += consumed
    if d.halo_depth > 1 and d.preconditioner == "jac_block":
        raise ValueError("read_input: Unable to use nonstandard halo depth with block jacobi preconditioner")
    return d


def write_deck(d: Deck) -> str:
    """Emit a deck the reference's reader accepts."""
    out = ["*tea"]
    for i, s in enumerate(d.states, start=1):
        line = "state %d density=%r energy=%r" % (i, s.density, s.energy)
        if i > 1:
            g = GEOMETRY_NAMES[s.geometry]
            line += " geometry=%s" % g
            if s.geometry == 2:
                line += " xmin=%r ymin=%r radius=%r" % (s.xmin, s.ymin, s.radius)
            elif s.geometry == 3:
                line += " xmin=%r ymin=%r" % (s.xmin, s.ymin)
            else:
                line += " xmin=%r xmax=%r ymin=%r ymax=%r" % (s.xmin, s.xmax, s.ymin, s.ymax)
        out.append(line)
    out += [
        "x_cells=%d" % d.x_cells,
        "y_cells=%d" % d.y_cells,
        "xmin=%r" % d.xmin,
        "ymin=%r" % d.ymin,
        "xmax=%r" % d.xmax,
        "ymax=%r" % d.ymax,
        "initial_timestep=%r" % d.initial_timestep,
        "end_step=%d" % d.end_step,
        "tl_max_iters=%d" % d.max_iters,
        "tl_use_%s" % d.solver,
        "tl_eps %r" % d.eps,
        "tl_preconditioner_type %s" % d.preconditioner,
        "tl_coefficient_%s" % ("inverse_density" if d.coefficient == RECIP_CONDUCTIVITY else "density"),
        "tl_ch_cg_presteps %d" % d.ch_cg_presteps,
        "tl_ch_cg_epslim %r" % d.ch_cg_epslim,
        "halo_depth %d" % d.halo_depth,
        "summary_frequency %d" % d.summary_frequency,
    ]
    if d.ppcg_inner_steps != -1:
        out.append("tl_ppcg_inner_steps %d" % d.ppcg_inner_steps)
    if d.reflective_boundary:
        out.append("reflective_boundary")
    if d.check_result:
        out.append("tl_check_result")
    if d.test_problem:
        out.append("test_problem %d" % d.test_problem)
    out.append("*endtea")
    return "\n".join(out) + "\n"


class SplitMix64:
    """SplitMix64 stream (Steele, Lea & Flood 2014) with uniform doubles from the top 53 bits."""

    MASK = (1 << 64) - 1

    def __init__(self, seed: int):
        self.state = seed & self.MASK

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & self.MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.MASK
        return z ^ (z >> 31)

    def uniform(self, lo: float, hi: float) -> float:
        u = (self.next_u64() >> 11) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u


def seeded_deck(
    cells: int,
    n_rect: int,
    n_circ: int = 0,
    seed: int = 1,
    rect_density=(0.1, 1.0),
    rect_energy=(1.0, 25.0),
    steps: int = 10,
    max_iters: int = 5000,
    solver: str = "cg",
    eps: float = 1.0e-15,
    coefficient: int = RECIP_CONDUCTIVITY,
) -> Deck:
    """Synthetic problem on the 10x10 domain: ambient state (density 100, energy 1e-4),
    ``n_rect`` rectangles with sides U[0.5,3] and lower corner U[0, 10-side], then
    ``n_circ`` circles with radius U[0.2,1], centre U[r, 10-r], density 0.1, energy 25.
    Rectangle density/energy are U[lo,hi] unless lo == hi.  Draw order per rectangle:
    width, height, x0, y0, density, energy; per circle: radius, cx, cy."""
    rng = SplitMix64(seed)
    states = [State(density=100.0, energy=1.0e-4)]
    for _ in range(n_rect):
        wdt = rng.uniform(0.5, 3.0)
        hgt = rng.uniform(0.5, 3.0)
        x0 = rng.uniform(0.0, 10.0 - wdt)
        y0 = rng.uniform(0.0, 10.0 - hgt)
        den = rng.uniform(*rect_density) if rect_density[0] != rect_density[1] else rect_density[0]
        en = rng.uniform(*rect_energy) if rect_energy[0] != rect_energy[1] else rect_energy[0]
        states.append(State(density=den, energy=en, geometry=1, xmin=x0, xmax=x0 + wdt, ymin=y0, ymax=y0 + hgt))
    for _ in range(n_circ):
        r = rng.uniform(0.2, 1.0)
        cx = rng.uniform(r, 10.0 - r)
        cy = rng.uniform(r, 10.0 - r)
        states.append(State(density=0.1, energy=25.0, geometry=2, xmin=cx, ymin=cy, radius=r))
    return Deck(
        states=states,
        x_cells=cells,
        y_cells=cells,
        xmin=0.0,
        ymin=0.0,
        xmax=10.0,
        ymax=10.0,
        initial_timestep=0.004,
        end_step=steps,
        max_iters=max_iters,
        eps=eps,
        solver=solver,
        coefficient=coefficient,
        summary_frequency=steps,
    )


def config_deck(index: int, solver: Optional[str] = None, cells: Optional[int] = None, seed: Optional[int] = None) -> Deck:
    """The five synthetic configurations (1-based index):
    1: 256^2, 3 rectangles (density 0.1, energy 25), CG, 10 steps, max 5000 iterations;
    2: 4096^2, 8 rectangles (density U[0.1,1], energy U[1,25]), CG (or Jacobi), 10 steps;
    3: as 2 with PPCG (10 inner steps, 20 CG presteps) or Chebyshev (20 presteps);
    4: 2048^2, rectangles as 2 (adjoint problem), 10 steps;
    5: 8192^2, 16 rectangles + 4 circles, CG, 20 steps.
    All: 10x10 domain, dt 0.004, tl_eps 1e-15, reciprocal-density coefficient keyword.
    ``cells`` overrides the mesh size (for reduced-size parity runs)."""
    s = index if seed is None else seed
    if index == 1:
        d = seeded_deck(cells or 256, 3, 0, s, rect_density=(0.1, 0.1), rect_energy=(25.0, 25.0), steps=10,
                        max_iters=5000, solver=solver or "cg")
    elif index == 2:
        d = seeded_deck(cells or 4096, 8, 0, s, steps=10, max_iters=50000, solver=solver or "cg")
    elif index == 3:
        d = seeded_deck(cells or 4096, 8, 0, s, steps=10, max_iters=50000, solver=solver or "ppcg")
        d.ppcg_inner_steps = 10
        d.ch_cg_presteps = 20
    elif index == 4:
        d = seeded_deck(cells or 2048, 8, 0, s, steps=10, max_iters=50000, solver=solver or "cg")
    elif index == 5:
        d = seeded_deck(cells or 8192, 16, 4, s, steps=20, max_iters=50000, solver=solver or "cg")
    else:
        raise ValueError("config index must be 1..5")
    return d
