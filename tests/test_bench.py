"""bench.py's roofline arithmetic (CPU): the per-step compulsory bytes of the fixed formula
B_step = N_cells x (2P + P + 2G + T + C reads + 2P + T + C writes) and the per-kernel byte
model of the dominant kernel, against the figures the design states."""
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
import bench  # noqa: E402


def test_step_bytes_per_cell():
    # FP64: moist (P = 13, T = 11, C = 9) and dry (P = 7, T = 5, C = 8), all 8 bytes, G = 29
    assert bench.step_bytes_per_cell(7, False) == (117 + 46) * 8 == 1304.0
    assert bench.step_bytes_per_cell(1, False) == (92 + 27) * 8 == 952.0
    # split: the state at 8 B; grid copies, tendencies and carried stencil diagnostics at 4 B
    assert bench.step_bytes_per_cell(7, True) == 928.0


def test_dominant_kernel_bytes():
    # the tracer solver: FP64 old and new density, FP32 mirror, tendency and new mirror per
    # tracer; w old and new, rho_g, T, area_z, 1/volume; the sediment-heating planes
    assert bench.kernel_bytes_per_cell("ks_column_tracers", 7, True, 0.3) == 202.0


def test_measured_traffic_table_names_kernels_of_the_step():
    # every entry names a kernel of the split step (the labels of its per-launch trace)
    assert "ks_column_tracers" in bench.MEASURED_DRAM_BYTES_PER_CELL
    assert all(k.startswith("ks_") for k in bench.MEASURED_DRAM_BYTES_PER_CELL)
