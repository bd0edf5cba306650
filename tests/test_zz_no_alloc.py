"""gch_get_timestep_noalloc: the CFL timestep for host codes that cannot
allocate device memory (a driver with a fixed, pre-sized memory budget that
forbids hidden allocations, or one that owns every device buffer through its
own pool).  The caller owns the state and the output slots; the library's
only other memory is a fixed array compiled into it.  Checked through the C
ABI against gch_get_timestep on the same state, on two calls in a row (the
shared array must not carry anything from one call into the next), and on a
call whose step reaches the next output time (dt clipped, dump flag set).

This file is named so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

from guacho_gb300 import params as P
from guacho_gb300 import problems

pytestmark = pytest.mark.gpu


def _noalloc(lib, p, u_dev_ptr, it, n_iter, t, tprint, dt_ptr, dump_ptr):
    from guacho_gb300 import _abi
    f = lib.gch_get_timestep_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(_abi.Params_t), C.c_void_p, C.c_int, C.c_int, C.c_double,
                  C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    s = _abi.to_struct(p)
    return f(C.byref(s), u_dev_ptr, it, n_iter, t, tprint, dt_ptr, dump_ptr, None)


@pytest.mark.parametrize("case", ["turbulence", "blast", "hydro"])
def test_noalloc_timestep_matches_domain_timestep(gpu_lib, case):
    import torch
    from guacho_gb300.domain import Domain
    if case == "turbulence":
        p, u0 = problems.turbulence(24, seed=12)
    elif case == "blast":
        p, u0 = problems.blast(20, p_in=5.0)
    else:
        p, u0 = problems.orszag_tang(20, 20, 4)
        p = p.replace(mhd=False, riemann_solver=P.SOLVER_HLLC, enable_flux_cd=False)
        u0 = np.ascontiguousarray(u0[..., :5])
    p = p.replace(precision=P.FP64)
    with Domain(p) as d:
        d.init(u0)
        states, refs = [], []
        t = 0.0
        for it in (1, 2):
            # the state the reference entry point sees (ghosts filled)
            states.append(d.download())
            dt, dump = d.get_timestep(it, 10, t, 0.05)
            refs.append((dt, dump))
            d.tstep(dt)
            t += dt
    dev = torch.device("cuda", 0)
    out_dt = torch.zeros(1, dtype=torch.float64, device=dev)
    out_dump = torch.zeros(1, dtype=torch.int32, device=dev)
    t = 0.0
    got = []
    for it, (u, (dt_ref, dump_ref)) in enumerate(zip(states, refs), start=1):
        u_dev = torch.from_numpy(u).to(dev)
        torch.cuda.synchronize()
        st = _noalloc(gpu_lib, p, u_dev.data_ptr(), it, 10, t, 0.05, out_dt.data_ptr(),
                      out_dump.data_ptr())
        assert st == 0
        torch.cuda.synchronize()
        got.append((float(out_dt.item()), bool(out_dump.item())))
        # FP64 arithmetic in the reference's order on both paths: equal bits
        assert got[-1][0] == dt_ref, (got[-1][0], dt_ref)
        assert got[-1][1] == dump_ref
        t += dt_ref
    # a repeated call on the same state returns the same value again
    st = _noalloc(gpu_lib, p, torch.from_numpy(states[1]).to(dev).data_ptr(), 2, 10,
                  refs[0][0], 0.05, out_dt.data_ptr(), out_dump.data_ptr())
    torch.cuda.synchronize()
    assert st == 0 and float(out_dt.item()) == got[1][0]


def test_noalloc_rejects_oversized_box(gpu_lib):
    """A box needing more partial minima than the fixed array holds is
    refused before any launch."""
    import torch
    from guacho_gb300 import _abi
    p = problems.orszag_tang(16, 16, 4)[0].replace(nx=1024, ny=1024, nz=1024)
    dev = torch.device("cuda", 0)
    u = torch.zeros(8, dtype=torch.float64, device=dev)   # never read: refused first
    out_dt = torch.zeros(1, dtype=torch.float64, device=dev)
    out_dump = torch.zeros(1, dtype=torch.int32, device=dev)
    st = _noalloc(gpu_lib, p, u.data_ptr(), 1, 10, 0.0, 1.0, out_dt.data_ptr(),
                  out_dump.data_ptr())
    assert st == _abi.ERR_TOO_LARGE


def test_noalloc_clips_to_output_time(gpu_lib):
    """current_time + dt >= tprint: dt is clipped to tprint - current_time
    and the dump flag is set (src/hydro_core.f90:691-694), as in
    gch_get_timestep on the same state."""
    import torch
    from guacho_gb300.domain import Domain
    p, u0 = problems.turbulence(24, seed=12)
    p = p.replace(precision=P.FP64)
    t = 0.125
    with Domain(p) as d:
        d.init(u0)
        u = d.download()
        dt_free, dump_free = d.get_timestep(20, 10, t, 1e30)
        assert not dump_free
        tprint = t + 0.5 * dt_free
        dt_ref, dump_ref = d.get_timestep(20, 10, t, tprint)
    assert dump_ref and dt_ref == tprint - t
    dev = torch.device("cuda", 0)
    out_dt = torch.zeros(1, dtype=torch.float64, device=dev)
    out_dump = torch.zeros(1, dtype=torch.int32, device=dev)
    u_dev = torch.from_numpy(u).to(dev)
    torch.cuda.synchronize()
    for _ in range(2):
        st = _noalloc(gpu_lib, p, u_dev.data_ptr(), 20, 10, t, tprint, out_dt.data_ptr(),
                      out_dump.data_ptr())
        torch.cuda.synchronize()
        assert st == 0
        assert float(out_dt.item()) == dt_ref
        assert bool(out_dump.item()) is True
    # the same state without the clip gives the free dt again
    st = _noalloc(gpu_lib, p, u_dev.data_ptr(), 20, 10, t, 1e30, out_dt.data_ptr(),
                  out_dump.data_ptr())
    torch.cuda.synchronize()
    assert st == 0 and float(out_dt.item()) == dt_free and not bool(out_dump.item())
