"""The largest arrays: a state of 2^31 or more values, where the split kernels
switch to 64-bit element indices (the 32-bit instance cannot address it).

A direction-stage at row k reads rows k-2 .. k+2 only (z) or row k only (x),
so the top rows of a tall grid (64 columns, ~7.9 M rows, 17 GB per FP64 state
array) and a 64-row grid filled with the same values and background slice must
come out bit-identical away from the small grid's bottom wall: the first runs
the 64-bit-index kernels at addresses beyond 2^31 elements, the second the
32-bit ones."""
import pytest
import torch

from pyminiweather_gb300 import _native

pytestmark = pytest.mark.gpu

NX = 64
PITCH = NX + 4
NZ_BIG = (1 << 31) // (4 * PITCH) + 64  # 4 * (nz + 4) * (nx + 4) >= 2^31
NZ_SMALL = 64
MARGIN = 4  # rows next to the small grid's bottom wall that differ


def _fill_state(nz, dev):
    """(4, nz+4, nx+4) FP64 values as smooth functions of (variable, row, column)."""
    a = torch.empty((4, nz + 4, PITCH), dtype=torch.float64, device=dev)
    kk = torch.arange(nz + 4, device=dev, dtype=torch.float64).view(-1, 1)
    col = torch.arange(PITCH, device=dev, dtype=torch.float64).view(1, -1)
    amp = (1e-3, 0.5, 0.3, 0.2)  # rho', rho*u, rho*w, (rho*theta)'
    for q in range(4):  # one plane at a time keeps the temporaries at a plane's size
        a[q] = amp[q] * torch.sin(0.37 * col + 0.011 * kk + q) + 0.1 * amp[q] * torch.cos(0.05 * kk)
    return a


def _backgrounds(nz, dev):
    kc = torch.arange(nz + 4, device=dev, dtype=torch.float64)  # cell centres, halo-indexed
    ki = torch.arange(nz + 1, device=dev, dtype=torch.float64)  # interfaces
    rho_c = 1.0 + 1e-4 * torch.cos(1e-3 * kc)
    rho_i = 1.0 + 1e-4 * torch.cos(1e-3 * (ki + 0.5))
    hy_dens_theta_c = 300.0 * rho_c
    hy_dens_theta_i = 300.0 * rho_i
    hy_p_i = 27.5629410929725921310572974482 * hy_dens_theta_i ** 1.4
    return [t.contiguous() for t in (rho_c, hy_dens_theta_c, rho_i, hy_dens_theta_i, hy_p_i)]


def test_64bit_index_stages_match_small_grid():
    free, _ = torch.cuda.mem_get_info()
    need = 5 * 4 * PITCH * (NZ_BIG + 4) * 8  # three state arrays and the fill's temporaries
    if free < need:
        pytest.skip("needs %.1f GB of free device memory" % (need / 1e9))
    assert 4 * PITCH * (NZ_BIG + 4) >= (1 << 31)
    dev = torch.device("cuda", torch.cuda.current_device())
    dx = dz = 20.0
    dt = 0.05
    stream = _native.stream_handle(dev)
    bg_big = _backgrounds(NZ_BIG, dev)
    init_big, frc_big = _fill_state(NZ_BIG, dev), _fill_state(NZ_BIG, dev)
    frc_big[1:3] *= 0.9  # forcing differs from init
    # the small grid holds exactly the big grid's top rows and background slice
    init_small = init_big[:, -(NZ_SMALL + 4):].clone()
    frc_small = frc_big[:, -(NZ_SMALL + 4):].clone()
    bg_small = [b[-(NZ_SMALL + 4):].clone() for b in bg_big[:2]] + [b[-(NZ_SMALL + 1):].clone() for b in bg_big[2:]]
    out_big = torch.empty_like(init_big)
    out_small = torch.empty_like(init_small)
    for mode in (1, 0):  # split (64-bit-index instance here), then native
        for direction in (0, 1):
            for nz, ini, frc, out, bg in ((NZ_BIG, init_big, frc_big, out_big, bg_big),
                                          (NZ_SMALL, init_small, frc_small, out_small, bg_small)):
                out.fill_(0.0)
                _native.call("mw_dirstage_f64", NX, nz, dx, dz, dt, *[_native.ptr(b) for b in bg], None,
                             _native.ptr(ini), _native.ptr(frc), _native.ptr(out), dt / 2, direction, mode, 0,
                             stream)
            torch.cuda.synchronize()
            top_big = out_big[:, -(NZ_SMALL + 2):-2, 2:-2]  # interior rows of the top band
            top_small = out_small[:, 2:-2, 2:-2]
            assert torch.isfinite(top_small).all()
            assert torch.equal(top_big[:, MARGIN:], top_small[:, MARGIN:]), (mode, direction)
    del init_big, frc_big, out_big
    torch.cuda.empty_cache()
