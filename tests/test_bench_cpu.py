"""The bench's host-side arithmetic and the reference arm's contract, on
the CPU: the algorithmic byte model per launch (the canonical 4R + 24C per
evaluation: 476 MB at 128^3 in FP64, 238 MB in the mixed form on FP32
vectors), the roofline reduction over a profile, the FP32-vector rule, and
one converged solve of the reference arm (the oracle port) at 32^3 with its
JSON line."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_byte_model_per_evaluation():
    import bench
    N = 128
    NR, NC = N ** 3, N * N * (N // 2 + 1)
    assert bench.alg_bytes(N, False)["eval_model"] == 4 * 8 * NR + 24 * 16 * NC  # 476 MB
    assert bench.alg_bytes(N, True, 4)["eval_model"] == 4 * 4 * NR + 24 * 8 * NC  # 238 MB
    ab = bench.alg_bytes(N, True, 4)
    assert ab["z_phi_grad"] == 10 * 8 * NC + 4 * NR
    assert ab["y_fft_5fields"] == 10 * 8 * NC
    # the Hessian set-up reads the FP64 iterate whatever the vectors' width
    assert ab["z_hess"] == bench.alg_bytes(N, True, 8)["z_hess"]


def test_roofline_of_a_profile():
    import bench
    N = 64
    prof = {"z_phi_grad_f32": (10, 1.0), "y_fft_5fields_f32": (20, 0.4),
            "x_conv_fwd_f32": (10, 0.3), "z_phi_grad": (2, 5.0)}
    r = bench.roofline(prof, N, True, 1000.0, "measured", vec_bytes=4)
    ab = bench.alg_bytes(N, True, 4)
    assert r["kernel"] == "z_phi_grad"  # the FP32 entries only
    assert r["avg_launch_ms"] == pytest.approx(0.1)
    assert r["achieved"] == pytest.approx(ab["z_phi_grad"] / 1e-4 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 1000.0)
    # conv: one evaluation's canonical bytes per z_phi launch over the conv kernels' time
    assert r["conv_hbm_gbs"] == pytest.approx(ab["eval_model"] * 10 / 1.7e-3 / 1e9)
    assert set(r["by_kernel"]) == {"z_phi_grad", "y_fft_5fields", "x_conv_fwd"}


def test_fp32_vector_rule(monkeypatch):
    import bench
    monkeypatch.delenv("DEFT_F32_VECTORS", raising=False)
    assert bench.f32_vectors(128, False) and bench.f32_vectors(256, False)
    assert not bench.f32_vectors(96, False)      # Nz not 32 * 2^k
    assert not bench.f32_vectors(128, True)      # no preconditioner
    monkeypatch.setenv("DEFT_F32_VECTORS", "0")
    assert not bench.f32_vectors(128, False)


def test_reference_arm_line_at_32():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--N", "32",
                          "--steps", "1", "--warmup", "1"], cwd=ROOT, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads(out.stdout.strip().splitlines()[-1])
    assert d["impl"] == "reference" and d["unit"] == "s" and d["higher_is_better"] is False
    assert d["value"] > 0 and d["steps"] == 1 and d["config"]["grid"] == [32, 32, 32]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
