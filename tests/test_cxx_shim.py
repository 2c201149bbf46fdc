"""The header-only C++ shim (include/helfem_gb300/TwoDBasis.hpp): compiled
with g++ against the library, it must behave like the reference's classes
(same signatures, same exception types) and give the same numbers as the
C ABI used directly."""
import os
import subprocess

import numpy as np
import pytest

import helfem_gb300 as hg

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def build_shim(tmp_path):
    exe = str(tmp_path / "shim_check")
    libdir = os.path.dirname(hg.__file__)
    subprocess.check_call(["g++", "-O1", "-std=c++17", os.path.join(HERE, "cxx", "shim_check.cpp"),
                           "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lhelfem_gb300",
                           f"-Wl,-rpath,{libdir}", "-o", exe])
    return exe


def parse(out, key):
    for line in out.splitlines():
        if line.startswith(key):
            toks = line.split()
            return {toks[i]: float(toks[i + 1]) for i in range(len(key.split()), len(toks) - 1, 2)}
    raise AssertionError(f"{key} missing in {out}")


def test_shim_host_side(tmp_path):
    exe = build_shim(tmp_path)
    out = subprocess.run([exe, "host"], capture_output=True, text=True, check=True).stdout
    a = hg.Atom(4, [0.0, 0.5, 2.0, 8.0, 40.0], [0, 1], [0, 0], nnodes=9, host_only=True)
    assert abs(parse(out, "atomic")["trS"] - np.trace(a.overlap())) < 1e-12 * abs(np.trace(a.overlap()))
    d = hg.Diatomic(1, 1, 0.7, [0.0, 0.8, 2.0, 4.7], [0, 1, 1, 1], [0, 0, 1, -1], nnodes=9, host_only=True)
    assert abs(parse(out, "diatomic")["trS"] - np.trace(d.overlap())) < 1e-12 * abs(np.trace(d.overlap()))
    assert "logic_error: Primitive teis have not been computed!" in out
    s = hg.SadAtom(10, [0.0, 0.5, 2.0, 8.0, 40.0], 1, nnodes=9, host_only=True)
    nr = s.nrad
    T = s.kinetic()
    Tl = 0.5 * (T[nr:2 * nr, nr:2 * nr] - T[:nr, :nr])
    r = parse(out, "sadatom")
    assert r["nrad"] == nr
    assert abs(r["trS"] - np.trace(s.overlap()[:nr, :nr])) < 1e-12 * abs(r["trS"])
    assert abs(r["trTl"] - np.trace(Tl)) < 1e-12 * abs(r["trTl"])
    assert "sadatom logic_error: Primitive teis have not been computed!" in out


def numbers(out, prefix):
    """Values following 'name value' pairs on the line starting with prefix."""
    for line in out.splitlines():
        if line.startswith(prefix):
            toks = line.split()[1:]
            return {toks[i]: float(toks[i + 1]) for i in range(0, len(toks) - 1, 2)}
    raise AssertionError(f"{prefix} missing in {out}")


@pytest.mark.gpu
def test_shim_gpu(tmp_path):
    exe = build_shim(tmp_path)
    out = subprocess.run([exe, "gpu"], capture_output=True, text=True, check=True).stdout
    a = hg.Atom(4, [0.0, 0.5, 2.0, 8.0, 40.0], [0, 1], [0, 0], nnodes=9)
    i, j = np.meshgrid(np.arange(a.nbf), np.arange(a.nbf), indexing="ij")
    P = 1e-2 / (1.0 + i + j)
    r = numbers(out, "atomic trPJ")
    tj = r["trPJ"]
    assert abs(tj - np.sum(P * a.coulomb_host(P))) < 1e-12 * abs(tj)
    assert abs(r["trPK"] - np.sum(P * a.exchange_host(P))) < 1e-12 * abs(r["trPK"])
    d = hg.Diatomic(1, 1, 0.7, [0.0, 0.8, 2.0, 4.7], [0, 1, 1, 1], [0, 0, 1, -1], nnodes=9)
    i, j = np.meshgrid(np.arange(d.nbf), np.arange(d.nbf), indexing="ij")
    Pd = 1e-3 / (1.0 + i + j)
    rd = numbers(out, "diatomic trPJ")
    tjd = rd["trPJ"]
    assert abs(tjd - np.sum(Pd * d.coulomb_host(Pd))) < 1e-12 * abs(tjd)
    assert abs(rd["trPK"] - np.sum(Pd * d.exchange_host(Pd))) < 1e-12 * abs(rd["trPK"])
    rx = numbers(out, "diatomic-xc")
    H, _, exc, nel = d.xc_host(1, 7, Pd)
    assert abs(rx["trPH"] - np.sum(Pd * H)) < 1e-12 * abs(rx["trPH"])
    assert abs(rx["Exc"] - exc) < 1e-12 * abs(exc) and abs(rx["Nel"] - nel) < 1e-12 * abs(nel)
    Ha, Hb, exc2, _ = d.xc_host(101, 130, Pd, 0.5 * Pd)
    assert abs(rx["trPHa"] - np.sum(Pd * Ha)) < 1e-12 * abs(rx["trPHa"])
    assert abs(rx["trPbHb"] - np.sum(0.5 * Pd * Hb)) < 1e-12 * abs(rx["trPbHb"])
    assert abs(rx["Exc2"] - exc2) < 1e-12 * abs(exc2)
    assert "runtime_error" in out
    s = hg.SadAtom(10, [0.0, 0.5, 2.0, 8.0, 40.0], 1, nnodes=9)
    i, j = np.meshgrid(np.arange(s.nrad), np.arange(s.nrad), indexing="ij")
    Pc = [1e-2 / (1.0 + l + i + j) for l in range(2)]
    Pr = Pc[0] + Pc[1]
    rs = numbers(out, "sadatom trPJ")
    assert abs(rs["trPJ"] - np.sum(Pr * s.coulomb_host(Pr))) < 1e-12 * abs(rs["trPJ"])
    K = s.exchange_host(Pc)
    for l in range(2):
        assert abs(rs[f"trPK{l}"] - np.sum(Pc[l] * K[l])) < 1e-12 * abs(rs[f"trPK{l}"])
    H, _, exc_s, _ = s.xc_host(1, 7, Pr)
    assert abs(rs["trPH"] - 4 * np.pi * np.sum(Pr * H)) < 1e-12 * abs(rs["trPH"])
    assert abs(rs["Exc"] - exc_s) < 1e-12 * abs(exc_s)
