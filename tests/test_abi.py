"""The drop-in boundary without a GPU: the C-ABI library loads and exports
every entry point include/usx_cu.h declares, the ctypes descriptors match the
C layouts, the `_usx` module imports with the reference's names, and compute
calls fail loudly (no CPU fallback) when no device is present."""

from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from conftest import HAVE_GPU, PKG, ROOT

HEADER = ROOT / "include" / "usx_cu.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(usx_cu_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("usx_cu_simulate", "usx_cu_demodulate", "usx_cu_bf_plan_create", "usx_cu_bf_execute",
                 "usx_cu_envelope", "usx_cu_color_flow", "usx_cu_axial_displacement", "usx_cu_axial_strain",
                 "usx_cu_scan_convert"):
        assert must in names


def test_library_exports_every_declared_symbol():
    so = PKG / "lib" / "libusx_cu.so"
    assert so.exists(), "libusx_cu.so is not built"
    lib = C.CDLL(str(so))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"
    assert lib.usx_cu_abi_version() == 1


def test_library_is_built_for_sm103a_only():
    """The build compiles device code for one target, sm_103a (no PTX for a
    JIT fallback, no other architecture)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("usx_build", PKG / "build.py")
    B = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(B)
    gencodes = re.findall(r"-gencode[= ]arch=(\w+),code=(\w+)", B.ARCH)
    assert gencodes == [("compute_103a", "sm_103a")], gencodes
    assert "-arch" not in B.ARCH and "compute_103a" not in gencodes[0][1]


@pytest.mark.gpu
def test_loaded_device_code_is_sm103():
    """At run time the loaded kernels are sm_103 code (cudaFuncGetAttributes)."""
    from usx import capi
    v = C.c_int(0)
    capi.check(capi.lib().usx_cu_binary_version(C.byref(v)), "usx_cu_binary_version")
    assert v.value == 103


def test_descriptor_layouts_match_header(tmp_path):
    """sizeof/offsetof of the C structs equal the ctypes mirrors."""
    from usx import capi
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "usx_types.h"\n'
                   "int main(){printf(\"%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n\","
                   "sizeof(usx_probe),sizeof(usx_medium),sizeof(usx_acquisition),sizeof(usx_transmit),"
                   "sizeof(usx_channel_desc),sizeof(usx_grid_desc),sizeof(usx_beamformer_config),"
                   "sizeof(usx_demod_config),sizeof(usx_simulator_config),sizeof(usx_doppler_config),"
                   "sizeof(usx_scatterer));return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    sizes = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    mirrors = [capi.Probe, capi.Medium, capi.Acquisition, capi.Transmit, capi.ChannelDesc, capi.GridDesc,
               capi.BeamformerConfig, capi.DemodConfig, capi.SimulatorConfig, capi.DopplerConfig]
    assert sizes[:10] == [C.sizeof(m) for m in mirrors]
    assert sizes[10] == 32


def test_module_surface_matches_reference_names():
    import usx
    for name in ("Simulator", "ImagingPipeline", "envelope", "Beamformer", "demodulate", "color_flow",
                 "estimate_axial_displacement", "axial_strain", "scan_convert", "log_compress", "apply_tgc",
                 "power_doppler", "apply_wall_filter", "design_lowpass", "compute_transmit_delays",
                 "transmit_arrival_time", "transmit_sensitivity", "element_directivity", "Phantom", "ScanGrid",
                 "ChannelData", "Frame", "angles_deg", "to_bmode", "grid_for", "extent_mm"):
        assert hasattr(usx, name), name
    assert usx.__backend__ == "cuda-sm_103a"


@pytest.mark.skipif(HAVE_GPU, reason="checks the behaviour without a GPU")
def test_compute_without_gpu_fails_loudly():
    import usx
    p = usx.presets.linear_5mhz()
    sim = usx.Simulator(p, usx.Medium(), usx.presets.acquisition(p, depth=0.02))
    with pytest.raises(RuntimeError, match="no CPU path"):
        sim.simulate(sim.make_plane_waves([0.0]), usx.Phantom.point_targets([usx.Vec3(0, 0, 0.01)]))


def test_validation_maps_to_value_error():
    """std::invalid_argument in the reference is ValueError here, raised on
    the host before any device work."""
    import usx
    cfg = usx.BeamformerConfig()
    cfg.mv_subarray = 1
    with pytest.raises(ValueError, match="mv_subarray"):
        usx.Beamformer(cfg)
    p = usx.Probe()
    p.element_width = 2 * p.pitch
    with pytest.raises(ValueError, match="overlap"):
        usx.Simulator(p, usx.Medium(), usx.Acquisition())
    with pytest.raises(ValueError):
        usx.ScanGrid.cartesian(0, 1, 0, 0, 1, 4)


def test_launch_shape_table_without_gpu():
    """The autotuner's launch-shape table is host metadata: 24 shapes in five
    kernel families, variant 0 the default thread-per-pixel shape, the
    channel-warp family (kind 4) with 4 pixel warps x 4 channel warps among
    them, and an index past the table rejected."""
    from usx import capi
    v = capi.das_variants()
    assert len(v) == 24
    assert v[0] == (8, 4, 8, 1, 0, 0)
    assert sorted({x[5] for x in v}) == [0, 1, 2, 3, 4]
    assert (4, 4, 0, 4, 0, 4) in v      # das_export_kernel / das_csum_kernel <4, 4, 4, 4>
    assert any(x[4] == 1 for x in v)    # deepest depth tiles first
    lib = capi.lib()
    kind = C.c_int(-1)
    assert lib.usx_cu_bf_variant_kind(len(v), C.byref(kind)) != 0
