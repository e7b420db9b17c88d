"""Image parity at the image configurations' own sizes: the GPU render against
the CPU restatement's render on the same sampler seed, judged against the CPU
render's own run-to-run noise at equal spp.

For each configuration the CPU restatement (oracle/pt_oracle.c, the path tracer
around the reference medium) renders with sampler seed A and with seed B, the GPU
with seed A; the bar is RMSE(GPU_A, CPU_A) <= RMSE(CPU_A, CPU_B), i.e. the GPU
image is no further from the CPU image than a second CPU render is.

* 256 x 256, 16 spp, 4 bounces: the sphere field with 3D noise and Renewal,
  Lambert albedo 0.8 (the full image).
* 1024 x 1024, 256 spp, 8 bounces: the nonstationary three-octave torus-plane
  field with 1D noise and Renewal+, a copper conductor with 1D NEE; the GPU
  renders the full image, the CPU two full-width rows through its middle at the
  full spp (a full CPU render takes hours), compared on those rows.
"""
import numpy as np
import pytest

from gpis_extend_gb300 import workloads
from oracle import oracle

pytestmark = pytest.mark.gpu


def rmse(a, b):
    return float(np.sqrt(np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2)))


def test_gpu_image_256_16spp_within_cpu_noise():
    from gpis_extend_gb300 import build, runtime
    build.build()
    desc = workloads.render_medium("sphere_3d")
    sc_a = workloads.render_scene(width=256, height=256, spp=16, max_bounces=4, sampler_seed=7)
    sc_b = workloads.render_scene(width=256, height=256, spp=16, max_bounces=4, sampler_seed=8)
    with runtime.Context(desc) as ctx:
        g_a, _ = ctx.render(sc_a)
    c_a, _ = oracle.render(desc, sc_a)
    c_b, _ = oracle.render(desc, sc_b)
    e_gpu, e_cpu = rmse(g_a, c_a), rmse(c_a, c_b)
    same = np.all(g_a == c_a, axis=2).mean()
    print(f"256^2 16 spp: RMSE(GPU_A, CPU_A) = {e_gpu:.3e}, RMSE(CPU_A, CPU_B) = {e_cpu:.3e}, "
          f"identical pixels {same:.4f}")
    assert e_cpu > 0.0
    assert e_gpu <= e_cpu


def test_gpu_image_1024_256spp_band_within_cpu_noise():
    from gpis_extend_gb300 import build, runtime
    build.build()
    desc = workloads.render_medium("torus_oct_nee")
    kw = dict(width=1024, height=1024, spp=256, max_bounces=8, phase="conductor", box_half=2.0)
    sc_a = workloads.render_scene(sampler_seed=7, **kw)
    sc_b = workloads.render_scene(sampler_seed=8, **kw)
    row0, rows = 511, 2
    with runtime.Context(desc) as ctx:
        g_a, _ = ctx.render(sc_a)
    c_a, _ = oracle.render_band(desc, sc_a, row0, rows)
    c_b, _ = oracle.render_band(desc, sc_b, row0, rows)
    g_band = g_a[row0:row0 + rows]
    e_gpu, e_cpu = rmse(g_band, c_a), rmse(c_a, c_b)
    same = np.all(g_band == c_a, axis=2).mean()
    print(f"1024^2 256 spp rows {row0}-{row0 + rows - 1}: RMSE(GPU_A, CPU_A) = {e_gpu:.3e}, "
          f"RMSE(CPU_A, CPU_B) = {e_cpu:.3e}, identical pixels {same:.4f}")
    assert e_cpu > 0.0
    assert e_gpu <= e_cpu
