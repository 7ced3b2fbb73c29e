"""The mixed-precision sweep policy (MixedSweeps in cc_ground.cpp) on synthetic residual
trajectories, on the CPU: split sweeps until the norm reaches the split floor or stalls
twice in a row, then FP64 record sweeps whose sliced products carry only the digits their
anchor needs (6 for an anchor the deltas leave at 1e4 x R_CONVERGENCE, 8 for one they
carry to R_CONVERGENCE, 9 for a confirmation or after a stall), delta sweeps in between,
and the end only on a 9-digit record sweep below R_CONVERGENCE.  A small C++ program is
compiled against the library's headers and linked to the built library."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def policy_lines(tmp_path_factory):
    from ugacc_gb300.build import build

    build()
    cxx = shutil.which("g++")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if not cxx or not os.path.isdir(cuda_inc):
        pytest.skip("needs g++ and the CUDA headers")
    libdir = os.path.join(ROOT, "ugacc_gb300", "lib")
    exe = str(tmp_path_factory.mktemp("policy") / "sweep_policy_check")
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "ugacc_gb300", "csrc"), "-I", cuda_inc,
                    os.path.join(ROOT, "tests", "cpp", "sweep_policy_check.cc"), "-L", libdir, "-lugacc_gb300",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return dict(line.split(":", 1) for line in out.strip().splitlines())


def test_mp2_start_at_no32_nv320(policy_lines):
    # 8 split sweeps, a 6-digit hand-over anchor, 3 deltas, an 8-digit re-anchor below
    # 1e4 x R_CONVERGENCE, 4 deltas, the 9-digit confirmation: the sequence measured on GPU
    assert policy_lines["mp2"].split() == (["split"] * 8 + ["record:6"] + ["delta"] * 3 + ["record:8"] +
                                           ["delta"] * 4 + ["record:9", "done"])


def test_one_slow_split_sweep_does_not_hand_over(policy_lines):
    assert policy_lines["guess"].split() == ["split"] * 6


def test_two_slow_split_sweeps_hand_over(policy_lines):
    # 5e-3 halves 0.1 (not slow); 4e-3 and 3.5e-3 do not halve their predecessors
    assert policy_lines["stall"].split() == ["split"] * 5 + ["record:6"]


def test_stalled_deltas_re_anchor_with_all_digits(policy_lines):
    # the deltas 9e-6 and 8.5e-6 each stay above 0.7 of their predecessor
    assert policy_lines["dstall"].split() == ["split", "split", "record:6", "delta", "delta", "delta", "record:9"]


def test_only_a_nine_digit_record_ends_the_solve(policy_lines):
    # R_CONVERGENCE 1e-7: the hand-over anchor needs 7 digits; its residual 5e-8 is below
    # R_CONVERGENCE, but the solve ends only on the 9-digit confirmation
    assert policy_lines["early"].split() == ["split", "split", "record:7", "record:9", "done"]
