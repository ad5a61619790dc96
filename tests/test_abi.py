"""The C-ABI library loads and exports every symbol include/apic_gpu.h declares
(no GPU compute here), and the host-only scene generators behave."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "apic_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\s*\*)\s+(apic_\w+)\s*\(", text, re.M)))


def test_every_declared_symbol_is_exported(gpu_lib):
    import apic_gb300
    syms = declared_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(gpu_lib, s), s
        assert s in apic_gb300.SIGNATURES, s


def test_no_device_fails_loudly(gpu_lib, has_gpu):
    import apic_gb300
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(apic_gb300.ApicError) as ei:
        apic_gb300.Apic(64, 64, 1 / 64, apic_gb300.WorldProperties())
    assert ei.value.code == apic_gb300.ERR_NO_DEVICE


def test_scene_counts_and_determinism(gpu_lib):
    import apic_gb300 as A
    # dam break x < 0.4, y < 0.6 on 128^2 at 4 particles per cell: cells 1..50 x 1..76
    p = A.scene_params(A.SCENE_DAM_BREAK, 128, cell_size=1 / 128, sub=2, seed=0, fluid_x=0.4, fluid_y=0.6)
    px, py, vx, vy = A.generate_scene(p)
    assert len(px) == 50 * 76 * 4
    px2, py2, _, _ = A.generate_scene(p)
    assert np.array_equal(px, px2) and np.array_equal(py, py2)
    assert np.all(vx == 0) and np.all(vy == 0)
    # every particle sits inside its own sub-cell of a non-border cell
    cx = np.floor(px * 128).astype(int)
    cy = np.floor(py * 128).astype(int)
    assert cx.min() >= 1 and cy.min() >= 1 and cx.max() <= 50 and cy.max() <= 76
    p3 = A.scene_params(A.SCENE_DAM_BREAK, 128, cell_size=1 / 128, sub=2, seed=1, fluid_x=0.4, fluid_y=0.6)
    assert not np.array_equal(px, A.generate_scene(p3)[0])


def test_scene_disk_and_noise(gpu_lib):
    import apic_gb300 as A
    p = A.scene_params(A.SCENE_DAM_BREAK_DISK, 256, cell_size=1 / 256, sub=2, seed=1, fluid_x=0.5, fluid_y=0.5,
                       disk=(0.7, 0.8, 0.08), disk_v=(0.0, -2.0))
    px, py, vx, vy = A.generate_scene(p)
    moving = vy == np.float32(-2.0)
    assert moving.sum() > 0
    assert np.all(np.hypot(px[moving] - 0.7, py[moving] - 0.8) < 0.08 + 2 / 256)
    q = A.scene_params(A.SCENE_NOISE, 128, cell_size=1 / 128, sub=2, seed=2, noise_period=0.1,
                       noise_threshold=0.5, vel_sigma=0.5)
    qx, qy, qvx, qvy = A.generate_scene(q)
    assert 0.1 * 126 * 126 * 4 < len(qx) < 0.9 * 126 * 126 * 4
    assert abs(float(np.std(qvx)) - 0.5) < 0.05 and abs(float(np.mean(qvy))) < 0.05


def test_reference_default_scene_generator_matches_oracle(gpu_lib, oracle_mod):
    import apic_gb300 as A
    o = oracle_mod.OracleSim(64, 64, 1 / 64, A.WorldProperties())
    n = o.info().num_particles
    px, py, _, _ = A.generate_scene(A.scene_params(A.SCENE_REFERENCE_DEFAULT, 64, cell_size=1 / 64))
    assert len(px) == n
    assert np.array_equal(o.read_field("pos_x")[:n], px)
    assert np.array_equal(o.read_field("pos_y")[:n], py)


def test_server_host_logic_without_device(gpu_lib, has_gpu):
    """Server bookkeeping on the host: modes, budget rejection, and a request
    whose scene cannot be created (no device here) fails instead of hanging."""
    import apic_gb300 as A
    if has_gpu:
        pytest.skip("a GPU is present")
    props = A.WorldProperties()
    sc = A.scene_params(A.SCENE_DAM_BREAK, 64, cell_size=1 / 64, sub=2, seed=0, fluid_x=0.5, fluid_y=0.5)
    with pytest.raises(A.ApicError) as ei:
        A.Server(1 << 20, 2).submit(A.scene_params(A.SCENE_DAM_BREAK, 256, cell_size=1 / 256, sub=2, seed=0,
                                                   fluid_x=0.7, fluid_y=0.7), props, 3, 1 / 240)
    assert ei.value.code == A.ERR_OOM
    for mode, threads in ((A.SERVER_CONTINUOUS, 2), (A.SERVER_CONTINUOUS, 0), (A.SERVER_ROUNDS, 0)):
        sv = A.Server(1 << 30, 2, mode=mode, prepare_threads=threads)
        with pytest.raises(A.ApicError):
            sv.set_mode(7, 1)
        ids = [sv.submit(sc, props, 2, 1 / 240) for _ in range(3)]
        for _ in range(50):
            rd = sv.step()
            assert rd.memory_used <= 1 << 30
            if rd.active == 0 and rd.queued == 0:
                break
        st = sv.stats()
        assert st.submitted == 3 and st.failed == 3 and st.completed == 0 and st.memory_used == 0
        assert st.mode == mode and st.prepare_threads == threads
        for rid in ids:
            info = sv.request(rid)
            assert info.finished and info.status == A.ERR_NO_DEVICE
        sv.close()


STRUCTS = {  # C struct of include/apic_gpu.h -> its ctypes mirror in apic_gb300
    "apic_world_props": "WorldPropsC", "apic_info": "InfoC", "apic_step_stats": "StatsC",
    "apic_scene_params": "SceneParamsC", "apic_server_round": "ServerRoundC", "apic_request_info": "RequestInfoC",
    "apic_batch_info": "BatchInfoC", "apic_server_stats": "ServerStatsC", "apic_render_params": "RenderParamsC",
    "apic_render_stats": "RenderStatsC",
}


def test_struct_layouts_match_the_header(tmp_path):
    """Every struct the C-ABI passes has the same size and field offsets in the
    header (compiled here with the host C compiler) as in the ctypes mirror."""
    import shutil
    import subprocess
    import apic_gb300 as A
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    text = open(os.path.join(ROOT, "include", "apic_gpu.h")).read()
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "apic_gpu.h"', "int main(void) {"]
    for c_name, py_name in STRUCTS.items():
        body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (c_name, c_name), text, re.S)
        assert body, c_name
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (c_name, c_name))
        for f, _ in getattr(A, py_name)._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (c_name, f, c_name, f))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        c_name, f, v = line.split()
        got[(c_name, f)] = int(v)
    for c_name, py_name in STRUCTS.items():
        cls = getattr(A, py_name)
        assert got[(c_name, "size")] == A.ctypes.sizeof(cls), c_name
        for f, _ in cls._fields_:
            assert got[(c_name, f)] == getattr(cls, f).offset, (c_name, f)
