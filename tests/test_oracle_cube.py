"""The oracle's restatement of critic2's NCI output against the reference's
own NCI cube/dat text (tests/golden/nci_cube_text.json, extracted from
tests/015_grdplot/ref/007_nciplot_mols-*): number formats, body layout and
the cutoff pass."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gold():
    with open(os.path.join(HERE, "golden", "nci_cube_text.json")) as f:
        return json.load(f)


def test_cube_number_format(oracle_mod, gold):
    """Every sampled body line of both cubes is reproduced exactly from its
    parsed numbers by the (" ",1p,e13.5e3) restatement."""
    for line in gold["dens_lines"] + gold["grad_lines"]:
        vals = [float(t) for t in line.split()]
        assert 1 <= len(vals) <= 6
        # a line with fewer than 6 numbers ends with the blank of the next item
        want = "".join(oracle_mod.fmt_e13(v) for v in vals) + (" " if len(vals) < 6 else "")
        assert want == line


def test_dat_number_format(oracle_mod, gold):
    for line in gold["dat_lines"]:
        a, b = (float(t) for t in line.split())
        assert oracle_mod.fmt_E15(a) + oracle_mod.fmt_E15(b) == line


def test_three_digit_exponents(oracle_mod):
    # Fortran's Ew.d drops the E for exponents beyond +-99
    assert oracle_mod.fmt_E15(1.25e-120) == "  1.2500000-120"
    assert oracle_mod.fmt_E15(-3.0e150) == " -3.0000000+150"
    assert oracle_mod.fmt_e13(1.25e-120) == "  1.25000E-120"
    assert oracle_mod.fmt_e13(0.0) == "  0.00000E+000"


def test_cube_body_layout(oracle_mod, gold):
    """Records of nstep(3) numbers, 6 a line: body line count and the
    length of every line."""
    n1, n2, n3 = gold["nstep"]
    assert gold["body_lines"] == n1 * n2 * ((n3 + 5) // 6)
    ns = np.array([2, 3, n3], np.int32)
    txt = oracle_mod.cube_body(ns, np.arange(2 * 3 * n3, dtype=float) + 0.5).decode()
    lines = txt.split("\n")[:-1]
    assert len(lines) == 2 * 3 * gold["lines_per_record"]
    per = [len(l) // 14 for l in lines[: gold["lines_per_record"]]]
    assert sum(per) == n3 and all(p == 6 for p in per[:-1])
    assert lines[gold["lines_per_record"] - 1].endswith(" ") == (n3 % 6 != 0)
    # the sampled reference lines have the same numbers per line at the same
    # positions within their records
    lpr = gold["lines_per_record"]
    for idx, line in zip(gold["sample_line_index"], gold["dens_lines"]):
        want = 6 if idx % lpr < lpr - 1 else n3 - 6 * (lpr - 1)
        assert len(line.split()) == want


def test_cutoff_pass_relation(gold):
    """In the reference's cubes s was set to 100 wherever the density cube
    reads |sign(lambda2) rho * 100| > 10 (rhoplot 0.1), and kept elsewhere
    (those points all have s < 100 in this grid)."""
    for ld, lg in zip(gold["dens_lines"], gold["grad_lines"]):
        for d, g in zip((float(t) for t in ld.split()), (float(t) for t in lg.split())):
            if abs(d) > 10.0 * (1 + 1e-5):
                assert g == 100.0
            elif abs(d) < 10.0 * (1 - 1e-5):
                assert g < 100.0


def test_nci_post_restatement(oracle_mod):
    """The oracle's cutoff pass on a synthetic cube: dat selection, order
    and the s := 100 rules."""
    rng = np.random.default_rng(0)
    ns = np.array([3, 4, 5], np.int32)
    n = int(ns.prod())
    crho = rng.uniform(-30, 30, n)
    cgrad = rng.uniform(0, 3, n)
    cg, dat = oracle_mod.nci_post(ns, crho, cgrad)
    sel = (np.abs(crho) < 20) & (cgrad < 2)
    assert np.array_equal(dat[:, 0], crho[sel] / 100) and np.array_equal(dat[:, 1], cgrad[sel])
    assert np.array_equal(cg, np.where(np.abs(crho) > 10, 100.0, cgrad))
    cg2, _ = oracle_mod.nci_post(ns, crho, cgrad, onlyneg=True, srho=(-0.05, 1.0))
    assert np.all(cg2[(crho > 0) | (crho < -5)] == 100.0)


def test_precise_cube_format(oracle_mod, gold):
    """writegrid_cube's E22.14E3 text: the sampled body lines and the header
    numbers of the reference's tests/005_plot cubes are reproduced exactly."""
    for name, c in gold["precise_cubes"].items():
        n3 = c["nstep"][2]
        assert c["body_lines"] == c["nstep"][0] * c["nstep"][1] * ((n3 + 5) // 6)
        for line in c["sample"]:
            vals = [float(t) for t in line.split()]
            want = "".join(" " + oracle_mod.fmt_E22(v) for v in vals) + (" " if len(vals) < 6 else "")
            assert want == line, name
        for line in c["header"][2:]:
            toks = line.split()
            nums = [float(t) for t in toks if "E" in t]
            for v in nums:
                assert oracle_mod.fmt_E22(v) in line
    assert oracle_mod.fmt_E22(0.0) == " 0.00000000000000E+000"
    assert oracle_mod.fmt_E22(-1.0) == "-0.10000000000000E+001"
