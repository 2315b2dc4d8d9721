"""The adjoint's binomial checkpoint schedule, on the CPU (no device needed).

``csrc/mol_adjoint.cu`` (``Adj::rev``) reverses steps [l, r) from the state u_l in its slot
with s spare slots: it advances ``checkpoint_split(r - l, s)`` steps (``csrc/mol_schedule.h``),
stores that state in a spare slot, reverses the right part with one spare slot fewer and then
the left part; with no spare slot it recomputes every state from l, and when every state of
[l, r) has a slot it stores them in one forward walk (r - l - 1 steps, what the split gives
there: one step per level).  A probe compiled with g++
against mol_schedule.h counts the forward steps of that recursion; they must equal the minimum
over all splits (a dynamic program here, for small cases) and Griewank's closed form
r n - C(c + r, r - 1) for the configurations' 64-snapshot adjoints.
"""
import math
import shutil
import subprocess
import sys
from functools import lru_cache

import pytest

ROOT = __file__.rsplit("/tests/", 1)[0]

PROBE = r"""
#include <cstdio>
#include <cstdlib>
#include <map>
#include <utility>
#include "mol_schedule.h"

static std::map<std::pair<long long, int>, long long> memo;

// forward steps Adj::rev advances for nn steps with `spare` spare slots
static long long advances(long long nn, int spare) {
    if (nn <= 1) return 0;
    if (spare == 0) return (nn - 1) * nn / 2;
    auto key = std::make_pair(nn, spare);
    auto it = memo.find(key);
    if (it != memo.end()) return it->second;
    const long long left = mol::checkpoint_split(nn, spare);
    if (left < 1 || left > nn - 1) { std::printf("bad split %lld %d %lld\n", nn, spare, left); std::exit(1); }
    const long long v = left + advances(nn - left, spare - 1) + advances(left, spare);
    memo[key] = v;
    return v;
}

int main(int argc, char** argv) {
    for (int i = 1; i + 1 < argc; i += 2) {
        const long long nn = std::atoll(argv[i]);
        const int spare = std::atoi(argv[i + 1]);
        std::printf("%lld\n", advances(nn, spare));
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    d = tmp_path_factory.mktemp("schedule")
    src = d / "probe.cpp"
    src.write_text(PROBE)
    exe = d / "probe"
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", f"{ROOT}/methodoflines.jl_gb300/csrc", "-o", str(exe), str(src)],
                   check=True)

    def run(cases):
        args = [str(v) for nn, s in cases for v in (nn, s)]
        out = subprocess.run([str(exe)] + args, check=True, capture_output=True, text=True).stdout.split()
        return [int(v) for v in out]
    return run


@lru_cache(maxsize=None)
def optimum(n, s):
    """Least forward steps over every split (s spare slots beside u_l's)."""
    if n <= 1:
        return 0
    if s == 0:
        return n * (n - 1) // 2
    return min(j + optimum(n - j, s - 1) + optimum(j, s) for j in range(1, n))


def revolve_minimum(n, c):
    """Griewank: r n - C(c + r, r - 1) with c checkpoints, r the least with C(c + r, r) >= n."""
    r = 0
    while math.comb(c + r, r) < n:
        r += 1
    return r * n - math.comb(c + r, r - 1)


def test_split_is_optimal_on_small_cases(probe):
    sys.setrecursionlimit(10000)
    cases = [(n, s) for n in range(2, 90) for s in range(1, 6)]
    got = probe(cases)
    for (n, s), g in zip(cases, got):
        assert g == optimum(n, s), (n, s, g, optimum(n, s))


def test_configuration_adjoints_take_griewanks_minimum(probe):
    # 64 slots: u_0's and 63 spare
    burgers, adr, few = probe([(20000, 63), (400, 63), (333, 1)])
    assert burgers == revolve_minimum(20000, 64) == 3 * 20000 - math.comb(67, 2) == 57789
    assert adr == revolve_minimum(400, 64) == 734
    assert few == revolve_minimum(333, 2) == 5400


def test_every_split_stays_inside_the_range(probe):
    # the probe exits non-zero on a split outside [1, nn - 1]
    probe([(nn, s) for nn in (2, 3, 1000, 123457) for s in (1, 2, 7, 63)] + [(10 ** 7, 63), (5000, 1000)])
