"""Snapshot (restart) files through the library against the files the
reference's own lb_io_write / field_io_write made from the same arrays
(tests/golden/io_*.npz, made by tests/golden/make_golden.py --only=io).

Written files must be byte-identical to the reference's; reading the
reference's files must give back the arrays it wrote (exactly for binary
records; ascii records hold 16 significant digits and must give the values
the text denotes).
"""

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["io_d1_phi_bin", "io_d2_phi_asc", "io_d1_q_asc", "io_d1_q_bin"]


def load(name):
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    g["names"] = [str(s) for s in g["files"]]
    return g


def objects(gb, g):
    L = tuple(int(v) for v in g["L"])
    ndist, nf = int(g["ndist"]), int(g["nf"])
    pe = gb.PE(0)
    cs = gb.Coords(pe, L)
    lb = gb.LB(cs, gb.FP64, ndist=ndist)
    fld = gb.Field(cs, nf, 2, gb.FP64, "q" if nf == 5 else "phi")
    hydro = gb.Hydro(cs, gb.FP64) if int(g["hydro"]) else None
    fmt = str(g["fmt"])
    lb.io_format(fmt, fmt)
    fld.io_format(fmt, fmt)
    if hydro:
        hydro.io_format(fmt, fmt)
    return (pe, cs), lb, fld, hydro, ndist


def put(lb, fld, hydro, g, ndist):
    lb.set(g["in_f"][:19])
    if ndist == 2:
        lb.set_g(g["in_f"][19:])
    fld.set(g["in_phi"])
    if hydro:
        hydro.set(rho=g["in_rho"], u=g["in_u"])


def ascii_values(buf):
    return np.array([float(w) for w in buf.decode().split()])


@pytest.mark.parametrize("name", CASES)
def test_write_matches_reference_bytes(gb, name, tmp_path, monkeypatch):
    g = load(name)
    keep, lb, fld, hydro, ndist = objects(gb, g)
    put(lb, fld, hydro, g, ndist)
    monkeypatch.chdir(tmp_path)
    lb.io_write(int(g["step"]))
    fld.io_write(int(g["step"]))
    if hydro:
        hydro.io_write(int(g["step"]))
    assert sorted(os.listdir(tmp_path)) == g["names"]
    for k, fn in enumerate(g["names"]):
        assert (tmp_path / fn).read_bytes() == g["file%d" % k].tobytes(), fn


@pytest.mark.parametrize("name", CASES)
def test_read_reference_files(gb, name, tmp_path, monkeypatch):
    g = load(name)
    keep, lb, fld, hydro, ndist = objects(gb, g)
    for k, fn in enumerate(g["names"]):
        (tmp_path / fn).write_bytes(g["file%d" % k].tobytes())
    monkeypatch.chdir(tmp_path)
    lb.io_read(int(g["step"]))
    fld.io_read(int(g["step"]))
    f = lb.get()
    if ndist == 2:
        f = np.concatenate([f, lb.get_g()])
    got = {fn.split("-")[0]: a for fn, a in (("dist", f), (fld.name, fld.get()))}
    want = {"dist": g["in_f"], fld.name: g["in_phi"]}
    if hydro:
        hydro.io_read(int(g["step"]))
        rho, u, _ = hydro.get()
        got.update(rho=rho, vel=u)
        want.update(rho=g["in_rho"], vel=g["in_u"])
    if str(g["fmt"]) == "binary":
        for k in want:
            assert np.array_equal(got[k], want[k]), k
        return
    # ascii: the values the reference's text denotes, in record order
    n = f[0].size
    for fn in g["names"]:
        if "metadata" in fn:
            continue
        stub = fn.split("-")[0]
        v = ascii_values(g["file%d" % g["names"].index(fn)].tobytes())
        a = got[stub]
        if stub == "dist":
            w = v.reshape(n, 19, ndist).transpose(2, 1, 0)
            assert np.array_equal(a.reshape(ndist, 19, n), w)
        else:
            w = v.reshape(n, -1).T
            assert np.array_equal(a.reshape(a.shape[0], n), w), stub


def test_fp32_state_round_trip(gb, tmp_path, monkeypatch):
    """A reduced-precision state goes out as the doubles of its values and
    comes back bit-identical; a restarted run continues exactly."""
    monkeypatch.chdir(tmp_path)
    L = (12, 10, 8)
    a = gb.BinaryFluid(L, gb.FP32, mobility=0.3, eta=0.1)
    a.phi.init_spinodal(8361235, 0.0, 0.02)
    a.step(20)
    a.lb.io_write(20)
    a.phi.io_write(20)
    a.hydro.io_write(20)              # u of the last step feeds the next
    b = gb.BinaryFluid(L, gb.FP32, mobility=0.3, eta=0.1)
    b.lb.io_read(20)
    b.phi.io_read(20)
    b.hydro.io_read(20)
    assert np.array_equal(a.lb.get(), b.lb.get())
    assert np.array_equal(a.phi.get(), b.phi.get())
    a.step(10)
    b.step(10)
    assert np.array_equal(a.phi.get(), b.phi.get())
    assert np.array_equal(a.lb.get(), b.lb.get())


def test_read_errors(gb, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    g = load("io_d1_phi_bin")
    keep, lb, fld, hydro, ndist = objects(gb, g)
    with pytest.raises(gb.LudwigGBError):
        lb.io_read(7)                                   # no such file
    # a file of another lattice size is rejected
    (tmp_path / "dist-000000007.001-001").write_bytes(b"\0" * 8 * 19 * 5)
    with pytest.raises(gb.LudwigGBError):
        lb.io_read(7)
