"""The algorithmic models behind bench.py's roofline figures, pinned to the padded-volume
byte model and the PSF FLOP model of the workloads (no GPU needed)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_byte_model_per_subiteration():
    import bench
    # 64^3, 8 angles per sub-iteration, attenuation: 91.77 MB
    fwd, bwd, sub = bench.alg_bytes_subiter(64, 8, 1)
    assert abs(sub / 1e6 - 91.77) < 0.01
    # 128^3, 12 angles per sub-iteration, attenuation: 1056.5 MB, 408 MB per forward launch
    fwd, bwd, sub = bench.alg_bytes_subiter(128, 12, 1)
    assert fwd == 408_145_920
    assert abs(sub / 1e6 - 1056.5) < 0.1


def test_psf_flop_model_of_the_128_cube_workload():
    from pytomography_gb300 import geometry, synthetic
    import bench
    w = synthetic.config2()
    n = w.shape[0]
    lp = n + 2 * geometry.compute_pad_size(n)
    sig = geometry.psf_sigma(lp, w.radius, w.dr[0], bench._PsfFit(w.psf))
    k = geometry.psf_kernel_size(sig, w.dr[0], 3.0)
    assert (lp, k) == (182, 29)
    per_angle = 2.0 * lp * lp * n * (2 * k)  # 2 P (K_r + K_z)
    assert abs(per_angle / 1e6 - 491.8) < 0.1


def test_reference_and_gpu_arms_share_the_config():
    import bench
    from pytomography_gb300 import synthetic
    w = synthetic.config2()
    a = bench.osem_config(w, 10, 12, 1)
    assert a == bench.osem_config(w, w.n_subsets, 12, 1)
    assert a["workload"] == "spect_128x128x128_120ang_att_psf" and a["parallelism"] == "single"
    assert bench.osem_config(w, 10, 12, 4)["parallelism"] == "replicas"
