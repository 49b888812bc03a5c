"""The reference's file formats through libwlc's host-side readers and
writers (no GPU): W<rank>.dat, M_OP<rank>.dat, RHO_total.dat, FreeEG.dat,
error.dat (SCFT_dump.f90:36-42,116-127,296-308; init_array_2dcomp_mod.f90:1088-1102)."""
import numpy as np

import wlc


def test_w_round_trip_is_exact(tmp_path):
    rng = np.random.default_rng(0)
    w = rng.normal(0.0, 3.0, size=(3, 250)) * 10.0 ** rng.integers(-8, 8, size=(3, 250))
    p = tmp_path / "W0.dat"
    wlc.io.write_w(p, w)
    assert np.array_equal(wlc.io.read_w(p, 250), w)
    first = p.read_text().splitlines()[0].split()
    assert int(first[0]) == 0 and len(first) == 4


def test_read_two_block_fortran_w_file(tmp_path):
    """A two-block W file as the reference writes it (list-directed K, WA, WB;
    D exponents and commas are accepted): w_C = 0."""
    p = tmp_path / "W0.dat"
    p.write_text("           0   1.2500000000000000       -3.0000000000000000D-02\n"
                 "           1,  2.0E+00, 4.5\n")
    w = wlc.io.read_w(p, 2)
    assert np.array_equal(w, np.array([[1.25, 2.0], [-0.03, 4.5], [0.0, 0.0]]))


def test_mop_round_trip_and_layout(tmp_path):
    rng = np.random.default_rng(1)
    a = rng.normal(size=(3, 3, 40))
    m = 0.5 * (a + a.transpose(1, 0, 2))
    p = tmp_path / "M_OP0.dat"
    wlc.io.write_mop(p, m, (4.0, 4.5, 5.0))
    lines = p.read_text().splitlines()
    assert len(lines) == 3 * 40
    # line a of point r: Lx Ly Lz M(r,a,0) M(r,a,1) M(r,a,2); m[b][a][r] = M(r, a, b)
    v = [float(x) for x in lines[3 * 7 + 1].split()]
    assert v[:3] == [4.0, 4.5, 5.0] and v[3:] == [m[0, 1, 7], m[1, 1, 7], m[2, 1, 7]]
    assert np.array_equal(wlc.io.read_mop(p, 40), m)


def test_rho_total_fixed_format(tmp_path):
    n = (4, 3, 2)
    nr = 24
    phi = np.random.default_rng(2).random((3, nr))
    p = tmp_path / "RHO_total.dat"
    wlc.io.write_rho(p, phi, n, (0.25, 0.5, 1.0))
    lines = p.read_text().splitlines()
    assert len(lines) == nr and all(len(ln) == 3 * 10 + 3 * 12 for ln in lines)
    # z outermost, x innermost; '(3f10.6,3f12.8)'
    ln = lines[1 * 12 + 2 * 4 + 3]  # z = 1, y = 2, x = 3
    r = 3 + 4 * (2 + 3 * 1)
    assert ln[:10] == "%10.6f" % 0.75 and ln[10:20] == "%10.6f" % 1.0 and ln[20:30] == "%10.6f" % 1.0
    assert ln[30:42] == "%12.8f" % phi[0, r] and ln[54:66] == "%12.8f" % phi[2, r]


def test_free_energy_and_error_logs(tmp_path):
    p = tmp_path / "FreeEG.dat"
    for it, fe in ((1, 3.5), (2, 3.25)):
        wlc.io.append_free_energy(p, it, fe, 0.5, 4.0, (15.0, 12.0, 18.0), (4, 2, 4), 10)
    lines = p.read_text().splitlines()
    assert len(lines) == 4
    fh = 15.0 * 0.4 * 0.2 + 12.0 * 0.4 * 0.4 + 18.0 * 0.2 * 0.4
    v = [float(x) for x in lines[2].split()]
    assert v[0] == 2 and v[1] == 3.25 and v[2] == 0.5 and v[3] == 3.75 and abs(v[4] - (3.25 - fh)) < 1e-15
    assert lines[3].split()[2] == "FE-FH"
    e = tmp_path / "error.dat"
    wlc.io.append_errors(e, 7, [1e-3, 2e-3, 3e-3, 0.0])
    assert [float(x) for x in e.read_text().split()] == [7.0, 1e-3, 2e-3, 3e-3, 0.0]


def test_missing_file_is_an_error(tmp_path):
    try:
        wlc.io.read_w(tmp_path / "nope.dat", 4)
    except wlc.WlcError as e:
        assert e.code == -8
    else:
        raise AssertionError("no error")
