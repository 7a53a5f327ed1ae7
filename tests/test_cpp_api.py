"""The C++ interfaces (include/vibe_gb300.hpp): a host program compiles and
links against the library here; on the GPU it runs and its results equal
those of the same calls made through the C ABI from Python."""
import os

import numpy as np
import pytest

import cpp_build


def test_cpp_api_compiles_and_links(tmp_path):
    if not os.path.exists(os.path.join(cpp_build.PKG, "libvibe_gb300.so")):
        pytest.skip("library not built")
    assert os.path.exists(cpp_build.build(str(tmp_path)))


@pytest.mark.gpu
def test_cpp_api_runs_and_matches_python(vg, tmp_path):
    import subprocess
    exe = cpp_build.build(str(tmp_path))
    out = tmp_path / "fields.bin"
    r = subprocess.run([exe, str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    data = np.fromfile(out, dtype=np.float64)
    s = vg.Setup.defaults(nx=20, ny=16, nz=12, dx=250.0, dy=250.0, z_top=3000.0, zeta_stretch=1.08,
                          bubble_xc=2500.0, bubble_yc=2000.0, bubble_zc=1000.0, bubble_radius_x=1500.0,
                          bubble_radius_z=1000.0, u_background=5.0, shear_u=0.001)
    with vg.Model(s, vg.FP64) as m, vg.Model(s, vg.FP64) as si:
        m.step(1.0, 4, 2)
        si.si_step(2.0, kind=vg.HZ_VERTICAL_TRIDIAGONAL)
        ref = np.concatenate([m.get(q) for q in range(7)] + [si.get(q) for q in range(7)])
    assert np.array_equal(data[:ref.size], ref)
    # the moist state stepped with the Kessler package through Integrator::set_physics
    mo = vg.Setup.defaults(**dict(s.as_dict(), moist=1, qv_surface=0.025, qv_decay_height=2500.0))
    with vg.Model(mo, vg.FP64) as w:
        w.set_physics_kessler(vg.Kessler.defaults(exner_offset=0))
        w.step(1.0, 4, 2)
        wet = np.concatenate([w.get(q) for q in (4, 6, 7, 8)])
    ncell = (s.nx + 8) * (s.ny + 8) * (s.nz + 8)  # the Helmholtz solution written before them
    tail = data[ref.size + ncell:ref.size + ncell + wet.size]
    assert np.array_equal(tail, wet)
    assert vg.interior(mo, 7, wet[2 * ncell:3 * ncell]).max() > 0.0  # the scheme condensed
    assert "dot test" in r.stdout
