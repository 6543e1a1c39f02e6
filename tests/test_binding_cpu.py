"""The reference-side binding (include/gpu_model.h) compiles against the
reference's own headers and links with its objects.

`make -C oracle binding` builds tests/binding/gpu_model_kat.cpp against the
reference checkout (CAFE_REFERENCE, or the oracle recipe's default) and
libcafe_gb300.so; the driver scores the reference's infer_processes
known-answer case (test.cpp:461-488, -lnL 46.56632) with the reference's
base_model and with gpu_base_model. Without a GPU the binding must fail
cleanly (std::runtime_error from cafe_ctx_create); with one, both values
agree to 1e-10. Skipped where the reference checkout is absent.
"""
import os
import subprocess

import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_gpu_model_binding_compiles_and_scores_the_reference_kat():
    ref = oracle.reference_dir()
    if ref is None:
        pytest.skip("no reference checkout (set CAFE_REFERENCE)")
    from cafe5_gb300 import build
    build.build()
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "binding", f"REF={ref}"], check=True,
                   capture_output=True, text=True, timeout=900)
    exe = os.path.join(ROOT, "oracle", "_ref", "gpu_model_kat")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    lines = dict(ln.split(" ", 1) for ln in r.stdout.strip().splitlines())
    reference = float(lines["reference"])
    # doctest::Approx(46.56632) in test.cpp
    assert abs(reference - 46.56632) < 1.2e-5 * (1 + 46.56632)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        assert r.returncode == 0, r.stdout + r.stderr
        assert abs(float(lines["gpu"]) - reference) <= 1e-10 * reference
    else:
        assert r.returncode == 3 and "gpu" in lines and lines["gpu"].startswith("unavailable"), r.stdout
