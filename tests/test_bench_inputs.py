"""The reference's field-benchmark input files (benches/main.rs:20-74):
the reader follows its text format, and the synthesized stand-ins have the
shapes its benchmarks expect (CPU test)."""
import numpy as np


def test_text_format_round_trip(gsc, tmp_path):
    from gstools_core import bench_inputs
    a1 = np.array([1.5, -2.25e-300, 3.0e10, 0.0])
    a2 = np.arange(12, dtype=np.float64).reshape(3, 4) / 7.0
    bench_inputs.write_1d(tmp_path / "a.txt", a1)
    bench_inputs.write_2d(tmp_path / "b.txt", a2)
    assert np.array_equal(bench_inputs.read_1d(tmp_path / "a.txt"), a1)
    got = bench_inputs.read_2d(tmp_path / "b.txt")
    assert got.shape == (3, 4) and np.array_equal(got, a2)
    # whitespace of any width, like split_whitespace (benches/main.rs:39-42)
    (tmp_path / "c.txt").write_text("1  2\t3\n4 5 6\n")
    assert np.array_equal(bench_inputs.read_2d(tmp_path / "c.txt"),
                          np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]]))


def test_synthesized_inputs_have_the_benchmark_shapes(gsc, tmp_path):
    from gstools_core import bench_inputs
    bench_inputs.synthesize_field_inputs(tmp_path, pos_no=500, mode_no=40, fourier_cut=3)
    a = bench_inputs.field_inputs(tmp_path)
    assert a["pos_2d"].shape == (2, 500) and a["pos_3d"].shape == (3, 500)
    assert a["cov_samples_2d"].shape == (2, 40) and a["cov_samples_3d"].shape == (3, 40)
    assert a["z_1"].shape == a["z_2"].shape == (40,)
    n = 7 * 7 - 1
    assert a["modes_2d"].shape == (2, n)
    assert a["spectrum_factor_2d"].shape == a["z_1_fourier"].shape == (n,)
    assert np.all(a["spectrum_factor_2d"] > 0)
    assert np.array_equal(a["pos_3d"][0], np.linspace(0.0, 10.0, 500))
