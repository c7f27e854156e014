"""CPU: the QMC integrators' lattices (include/gbint/qmc.hh, host code): the size ladder is
strictly increasing primes from 1021 with ratio ~1.09, next_n picks the smallest size >= the
request (the largest when none is), and the Korobov generating vectors are (1, a, a^2, ...) mod n
with a no worse under P_2 than the simple multipliers 2, 3, n/2, n/3, cached per (n, dimension).
"""
import os
import shutil
import subprocess

import pytest

from diffrg_gb300 import build as B

HERE = os.path.dirname(os.path.abspath(__file__))


def _is_prime(v):
    if v < 2:
        return False
    p = 2
    while p * p <= v:
        if v % p == 0:
            return False
        p += 1
    return True


@pytest.fixture(scope="module")
def out(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    cuda = os.path.dirname(os.path.dirname(B.nvcc()))
    exe = str(tmp_path_factory.mktemp("qmc") / "qmc_lattices")
    cmd = [gxx, "-std=c++20", "-O2", "-I", B.INCLUDE, "-I", os.path.join(cuda, "include"),
           "-I", os.path.join(cuda, "include", "cccl"), os.path.join(HERE, "cpp", "qmc_lattices.cc"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout.splitlines()


def test_size_ladder(out):
    f = next(l for l in out if l.startswith("SIZES")).split()
    first = [int(v) for v in f[2:f.index("LAST")]]
    last = int(f[f.index("LAST") + 1])
    assert first[0] == 1021 and all(_is_prime(v) for v in first)
    assert all(b > a for a, b in zip(first, first[1:]))
    assert all(1.05 < b / a < 1.13 for a, b in zip(first, first[1:]))
    assert 1e9 < last < 2 ** 31


def test_next_n(out):
    nx = {int(l.split()[1]): int(l.split()[2]) for l in out if l.startswith("NEXT")}
    assert nx[1] == 1021 and nx[512] == 1021 and nx[1021] == 1021 and nx[1022] > 1021
    assert nx[100000] >= 100000 and _is_prime(nx[100000])
    assert nx[5000000000] < 2 ** 31  # beyond the ladder: its largest size


def test_korobov_vectors(out):
    lats = [l.split() for l in out if l.startswith("LAT")]
    assert len(lats) == 9
    for _, dim, n, z0, z1, z2, z3, p2, worst, cached in lats:
        dim, n, z = int(dim), int(n), [int(z0), int(z1), int(z2), int(z3)]
        assert z[0] == 1 and int(cached) == 1
        if dim == 1:
            continue
        a = z[1]
        assert 2 <= a <= n - 2
        for j in range(2, dim):
            assert z[j] == z[j - 1] * a % n
        assert float(p2) <= float(worst)
