"""The allocation-free sensitivity entry point against the context-based one.

topo_sensitivity_rhs_noalloc serves callers that cannot allocate device
memory (for example hosts with a fixed memory pool, or loops that must not pay
cudaMalloc's device-wide synchronisation): it takes no context and uses a fixed scratch array
inside the library.  It must reproduce topo_sensitivity_rhs of a mixed
precision context on the same inputs, on consecutive calls (the shared
scratch keeps the previous call's contents), and refuse meshes larger than
its scratch.  The file name makes pytest collect it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX, NY = 40, 20


def _lib():
    from topomax_gb300 import _capi
    lib = _capi.load_library()
    f = lib.topo_sensitivity_rhs_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(_capi.GridDesc), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                  ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return lib, _capi


def _problem():
    import topomax_gb300 as tg
    from topomax_gb300.designs import parse_design_dict
    dom, par = parse_design_dict({"Elasticity": {
        "domain_parameters": dict(width=2.0, height=1.0, fem_step_size=0.002, dem_step_size=1.0,
                                  penalties=[3.0], volume_fraction=0.5),
        "problem_parameters": dict(fixed_sides=["Left"], body_force=None,
                                   tractions=[dict(side="Right", center=0.5, length=0.5, value=[0.0, -1.0])],
                                   filter_radius=0.05, young_modulus=1.0, poisson_ratio=0.3)}})
    mesh = tg.RectangleMesh(2.0, 1.0, NX, NY)
    V = tg.FunctionSpace(mesh, "CG", 1, dof_order="lattice")
    prob = tg.ElasticityProblem(mesh, V, dom, par, precision="mixed", rtol=1e-10)
    prob.set_penalization(3.0)
    return prob, V


def test_noalloc_matches_context_entry_point():
    import torch
    lib, capi = _lib()
    prob, V = _problem()
    rho = np.random.default_rng(5).uniform(0.05, 1.0, V.dim())
    prob.calculate_objective(rho)
    u, xi = prob.u.tensor, prob.filtered_rho.tensor
    ref = prob.sensitivity_rhs(prob.u, xi)
    torch.cuda.synchronize()
    grid = capi.GridDesc(2.0, 1.0, NX, NY)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    outs, free = [], []
    bufs = [torch.full_like(ref, float("nan")) for _ in range(2)]
    for b in bufs:   # consecutive calls share the scratch array
        rc = lib.topo_sensitivity_rhs_noalloc(ctypes.byref(grid), 1.0, 0.3, 3.0, 1e-6,
                                              ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(xi.data_ptr()),
                                              ctypes.c_void_p(b.data_ptr()), stream)
        assert rc == 0
        torch.cuda.synchronize()
        outs.append(b.clone())
        free.append(torch.cuda.mem_get_info()[0])
    # the CUDA runtime materialises the fixed scratch array when the library's device code
    # is first loaded; after that, calls take no device memory
    assert free[1] == free[0]
    scale = ref.abs().max().item()
    for b in outs:
        assert torch.isfinite(b).all()
        assert (b - ref).abs().max().item() <= 1e-12 * scale


def test_noalloc_rejects_meshes_beyond_its_scratch():
    import torch
    lib, capi = _lib()
    big = capi.GridDesc(2.0, 1.0, 1024, 513)     # 2*1024*513 > 2^20 triangles
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(dummy.data_ptr())
    rc = lib.topo_sensitivity_rhs_noalloc(ctypes.byref(big), 1.0, 0.3, 3.0, 1e-6, p, p, p,
                                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == capi.TOPO_ERR_ARG
