"""Deck reader/writer and the seeded problem generator (host logic, no GPU)."""
import numpy as np

from tealeaf_ref_gb300 import deck as dk


def test_parse_reference_decks(golden):
    d = dk.parse_deck(golden["benchmarks"]["tea_bm_4"]["deck"])
    assert (d.x_cells, d.y_cells) == (1000, 1000)
    assert d.solver == "cg" and d.max_iters == 10000 and d.eps == 1e-15
    assert d.initial_timestep == 0.004 and d.end_step == 10 and d.test_problem == 4
    assert len(d.states) == 5 and d.states[1].geometry == 1 and d.states[1].energy == 25.0
    p = dk.parse_deck(golden["ppcg_deck"])
    assert p.solver == "ppcg" and p.halo_depth == 2 and p.preconditioner == "none"
    assert p.effective_inner_steps() == 4 * int(np.sqrt(np.sqrt(np.float32(1e6))))


def test_defaults_follow_read_input():
    d = dk.parse_deck("*tea\nstate 1 density=1 energy=1\n*endtea\n")
    assert d.solver == "jacobi" and d.max_iters == 1000 and d.ch_cg_presteps == 25
    assert d.eps == float(np.float32(1e-10)) and d.ch_cg_epslim == 1.0 and d.halo_depth == 1
    assert d.coefficient == dk.CONDUCTIVITY and d.preconditioner == "none"


def test_comments_case_and_separators():
    text = """*TEA
STATE 1 DENSITY=2.5, ENERGY=3 ! ambient
state 2 density=1 energy=2 geometry=circle xmin=1 ymin=2 radius=0.5 ; circle
X_CELLS=8
y_cells 9
tl_use_chebyshev
tl_coefficient_inverse_density
reflective_boundary
tl_preconditioner_type jac_block
*ENDTEA
"""
    d = dk.parse_deck(text)
    assert d.states[0].density == 2.5 and d.states[0].energy == 3.0
    assert d.states[1].geometry == 2 and d.states[1].radius == 0.5
    assert (d.x_cells, d.y_cells) == (8, 9) and d.solver == "chebyshev"
    assert d.coefficient == dk.RECIP_CONDUCTIVITY and d.reflective_boundary
    assert d.preconditioner == "jac_block"


def test_writer_round_trip():
    for i in (1, 3, 5):
        d = dk.config_deck(i)
        e = dk.parse_deck(dk.write_deck(d))
        for f in ("x_cells", "y_cells", "solver", "max_iters", "eps", "coefficient", "end_step",
                  "initial_timestep", "ch_cg_presteps", "ppcg_inner_steps"):
            assert getattr(e, f) == getattr(d, f), f
        assert len(e.states) == len(d.states)
        for a, b in zip(e.states, d.states):
            assert a == b


def test_seeded_generator_is_deterministic():
    a = dk.config_deck(5)
    b = dk.config_deck(5)
    assert a.states == b.states
    assert len(a.states) == 1 + 16 + 4
    c = dk.config_deck(5, seed=6)
    assert c.states != a.states
    for s in a.states[1:17]:
        assert 0.5 <= s.xmax - s.xmin <= 3.0 and 0.0 <= s.xmin and s.xmax <= 10.0
        assert 0.1 <= s.density <= 1.0 and 1.0 <= s.energy <= 25.0
    for s in a.states[17:]:
        assert s.geometry == 2 and 0.2 <= s.radius <= 1.0 and s.density == 0.1


def test_splitmix64_known_values():
    # SplitMix64 with seed 0: first output is 0xE220A8397B1DCDAF (published test vector)
    g = dk.SplitMix64(0)
    assert g.next_u64() == 0xE220A8397B1DCDAF


def test_tiling_keywords_are_read():
    """The tiling keywords take a value (read_input.f90:175-184) and must not leave it behind
    as a stray word; use_fortran_kernels is a flag."""
    text = ("*tea\nstate 1 density=100.0 energy=0.0001\nx_cells 10\ny_cells 12\ntiles_per_problem 4\n"
            "sub_tiles_per_tile 2\nuse_fortran_kernels\ntl_max_iters 77\n*endtea\n")
    d = dk.parse_deck(text)
    assert (d.tiles_per_problem, d.sub_tiles_per_tile, d.use_fortran_kernels) == (4, 2, True)
    assert (d.x_cells, d.y_cells, d.max_iters) == (10, 12, 77)
