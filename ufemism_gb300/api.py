"""Python mirror of the reference interface for the ice-velocity solve.

``solve_SSA`` / ``solve_SIA`` of ice_dynamics_module.f90 take (mesh, ice) and update the ice
fields in place; here :class:`DeviceMesh` holds the uploaded mesh and ``solve_ssa`` /
``solve_sia`` take dicts of the same ``type_ice_model`` fields (same names, Aa arrays of nV
entries, Ac arrays of nAc, AaAc arrays of nVAaAc). All arithmetic runs in the CUDA library
through the C-ABI; nothing here computes a solve on the CPU.
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass, field

import numpy as np

from . import _native as nat

ZETA_DEFAULT = np.array([0.00, 0.10, 0.20, 0.30, 0.40, 0.50, 0.60, 0.70, 0.80, 0.90,
                         0.925, 0.95, 0.975, 0.99, 1.00])  # configuration_module.f90:124-126


def default_params(**kw) -> dict:
    """Solver knobs (configuration_module.f90:169-184) with the values the benchmark
    workloads use: Picard tolerance 1e-3, SOR omega 1.3, SOR tolerance 1e-4 m/yr,
    m_enh = 1, linear sliding with beta^2 = 1e3 Pa yr/m. Keywords override."""
    p = dict(SSA_RN_tol=1e-3, SSA_max_outer_loops=50, SSA_max_residual_UV=1e-4, SSA_SOR_omega=1.3,
             SSA_max_inner_loops=10000, m_enh_ssa=1.0, m_enh_sia=1.0,
             sliding_law=nat.UFE_SLIDING_LINEAR, beta_sq=1e3, use_analytical_GL_flux=0,
             zero_velocities=0, zeta=ZETA_DEFAULT, precision=nat.UFE_FP64, mixed_refold_sweeps=0,
             fp64_exact=0, mixed_fp32_viscosity=0)
    p.update(kw)
    return p


def _params_struct(p: dict):
    zeta = np.ascontiguousarray(p["zeta"], dtype=np.float64)
    s = nat.Params(p["SSA_RN_tol"], p["SSA_max_outer_loops"], p["SSA_max_residual_UV"], p["SSA_SOR_omega"],
                   p["SSA_max_inner_loops"], p["m_enh_ssa"], p["m_enh_sia"], p["sliding_law"], p["beta_sq"],
                   p["use_analytical_GL_flux"], p["zero_velocities"], zeta.size, zeta.ctypes.data,
                   p["precision"], p.get("mixed_refold_sweeps", 0), p.get("fp64_exact", 0),
                   p.get("mixed_fp32_viscosity", 0))
    return s, zeta


def _f64(a):
    return np.asfortranarray(a, dtype=np.float64)


def _i32(a):
    return np.asfortranarray(a, dtype=np.int32)


def _ptr(a):
    return None if a is None else a.ctypes.data


@dataclass
class AaAcMesh:
    """Base triangulation plus the Ac / AaAc mesh, neighbour functions and colouring, in the
    reference's layout (1-based index values, Fortran-order arrays)."""
    base: object
    nAc: int
    nVAaAc: int
    arrays: dict = field(default_factory=dict)

    def __getattr__(self, name):
        arrays = self.__dict__.get("arrays", {})
        if name in arrays:
            return arrays[name]
        raise AttributeError(name)


def build_aaac(base) -> AaAcMesh:
    """Ac mesh, combined AaAc mesh, neighbour functions and five-colouring of ``base``
    (make_Ac_mesh, get_neighbour_functions, calculate_five_colouring_AaAc) by the library's
    host mesh substrate."""
    L = nat.load()
    nV, nTri, ncm = base.nV, base.nTri, base.C.shape[1]
    nAc = nV + nTri - 1
    nA = nV + nAc
    z = lambda *s: np.zeros(s, dtype=np.float64, order="F")
    zi = lambda *s: np.zeros(s, dtype=np.int32, order="F")
    arr = dict(Nx=z(nV, ncm + 1), Ny=z(nV, ncm + 1), Nxx=z(nV, ncm + 1), Nxy=z(nV, ncm + 1), Nyy=z(nV, ncm + 1),
               iAci=zi(nV, ncm), Aci=zi(nAc, 4), VAc=z(nAc, 2), Nx_Ac=z(nAc, 4), Ny_Ac=z(nAc, 4), No_Ac=z(nAc, 4),
               Np_Ac=z(nAc), edge_index_Ac=zi(nAc), VAaAc=z(nA, 2), nCAaAc=zi(nA), CAaAc=zi(nA, ncm),
               Nx_AaAc=z(nA, ncm + 1), Ny_AaAc=z(nA, ncm + 1), Nxx_AaAc=z(nA, ncm + 1), Nxy_AaAc=z(nA, ncm + 1),
               Nyy_AaAc=z(nA, ncm + 1), colour=zi(nA), colour_vi=zi(nA, 5), colour_nV=zi(5))
    keep = dict(V=_f64(base.V), nC=_i32(base.nC), C=_i32(base.C), niTri=_i32(base.niTri), iTri=_i32(base.iTri),
                Tri=_i32(base.Tri), edge_index=_i32(base.edge_index))
    b = nat.BaseMeshC(nV, nTri, ncm, *(_ptr(keep[k]) for k in ("V", "nC", "C", "niTri", "iTri", "Tri", "edge_index")))
    o = nat.AaAcMeshC(nAc, nA, *(_ptr(arr[k]) for k in nat.AAAC_FIELDS))
    rc = L.ufe_aaac_build(ct.byref(b), ct.byref(o))
    if rc != nat.UFE_OK:
        raise nat.UfeError(rc, "ufe_aaac_build")
    return AaAcMesh(base=base, nAc=nAc, nVAaAc=nA, arrays=arr)


def init(device: int = 0) -> None:
    rc = nat.load().ufe_init(device)
    if rc != nat.UFE_OK:
        raise nat.UfeError(rc, "ufe_init")


def _mesh_desc(mesh):
    """ufe_mesh_desc of a mesh, with the arrays it points to (keep them alive until the
    library has copied them)."""
    base = mesh.base
    k = dict(V=_f64(base.V), nC=_i32(base.nC), iAci=_i32(mesh.iAci), Aci=_i32(mesh.Aci),
             edge_index=_i32(base.edge_index), edge_index_Ac=_i32(mesh.edge_index_Ac),
             nCAaAc=_i32(mesh.nCAaAc), CAaAc=_i32(mesh.CAaAc), Nx_AaAc=_f64(mesh.Nx_AaAc),
             Ny_AaAc=_f64(mesh.Ny_AaAc), Nxx_AaAc=_f64(mesh.Nxx_AaAc), Nxy_AaAc=_f64(mesh.Nxy_AaAc),
             Nyy_AaAc=_f64(mesh.Nyy_AaAc), colour=_i32(mesh.colour), colour_vi=_i32(mesh.colour_vi),
             colour_nV=_i32(mesh.colour_nV))
    d = nat.MeshDesc(base.nV, mesh.nAc, mesh.nVAaAc, k["CAaAc"].shape[1],
                     *(_ptr(k[n]) for n in ("V", "nC", "iAci", "Aci", "edge_index", "edge_index_Ac", "nCAaAc",
                                            "CAaAc", "Nx_AaAc", "Ny_AaAc", "Nxx_AaAc", "Nxy_AaAc", "Nyy_AaAc",
                                            "colour", "colour_vi", "colour_nV")))
    return d, k


def _ssa_in(fields: dict):
    keep = {}

    def g(k, dt=np.float64):
        v = fields.get(k)
        if v is None:
            return None
        a = np.ascontiguousarray(v, dtype=dt)
        keep[k] = a
        return a.ctypes.data

    ints = ("mask_sheet", "mask_gl_Ac")
    return nat.SsaIn(*(g(k, np.int32 if k in ints else np.float64) for k in nat.SSA_IN_FIELDS)), keep


SSA_INOUT_FIELDS = ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac", "N_AaAc")
SSA_OUT_FIELDS = ("Up_SSA_Ac", "Uo_SSA_Ac", "eta_AaAc", "S_AaAc", "tau_c_AaAc", "phi_fric_AaAc")


def _ssa_sizes(nV, nAc, nA) -> dict:
    sizes = {k: nA for k in SSA_INOUT_FIELDS + SSA_OUT_FIELDS}
    sizes.update(U_SSA=nV, V_SSA=nV, Ux_SSA_Ac=nAc, Uy_SSA_Ac=nAc, Up_SSA_Ac=nAc, Uo_SSA_Ac=nAc)
    return sizes


def ssa_buffers(nV, nAc, nA) -> dict:
    """Host arrays for the buffers= forms, zero (a cold start): the warm start that a solve
    overwrites with its solution (U_SSA, V_SSA, Ux_SSA_Ac, Uy_SSA_Ac, N_AaAc) and the other
    outputs — the model's own state arrays, kept across time steps."""
    return {k: np.zeros(n) for k, n in _ssa_sizes(nV, nAc, nA).items()}


def _check_buffers(buffers: dict, nV, nAc, nA):
    for k, n in _ssa_sizes(nV, nAc, nA).items():
        b = buffers.get(k)
        if not (isinstance(b, np.ndarray) and b.dtype == np.float64 and b.flags.c_contiguous and b.shape == (n,)):
            raise ValueError("buffers[%r] must be a contiguous float64 array of %d" % (k, n))


def _buffer_structs(buffers: dict):
    sio = nat.SsaInout(*(buffers[k].ctypes.data for k in SSA_INOUT_FIELDS))
    so = nat.SsaOut(*(buffers[k].ctypes.data for k in SSA_OUT_FIELDS))
    return sio, so


def _ssa_structs(nV, nAc, nA, fields: dict, warm: dict | None):
    si, keep = _ssa_in(fields)
    warm = warm or {}
    io = {}
    for k, n in (("U_SSA", nV), ("V_SSA", nV), ("Ux_SSA_Ac", nAc), ("Uy_SSA_Ac", nAc)):
        io[k] = np.array(warm.get(k, np.zeros(n)), dtype=np.float64, copy=True)
    io["N_AaAc"] = np.array(warm.get("N_AaAc", np.zeros(nA)), dtype=np.float64, copy=True)
    sio = nat.SsaInout(*(io[k].ctypes.data for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac", "N_AaAc")))
    return si, sio, io, keep


def _download_structs(nV, nAc, nA):
    io = {k: np.zeros(nV) for k in ("U_SSA", "V_SSA")}
    io.update({k: np.zeros(nAc) for k in ("Ux_SSA_Ac", "Uy_SSA_Ac", "Up_SSA_Ac", "Uo_SSA_Ac")})
    io.update({k: np.zeros(nA) for k in ("N_AaAc", "eta_AaAc", "S_AaAc", "tau_c_AaAc", "phi_fric_AaAc")})
    sio = nat.SsaInout(*(io[k].ctypes.data for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac", "N_AaAc")))
    so = nat.SsaOut(*(io[k].ctypes.data for k in ("Up_SSA_Ac", "Uo_SSA_Ac", "eta_AaAc", "S_AaAc", "tau_c_AaAc",
                                                   "phi_fric_AaAc")))
    return io, sio, so


class DeviceMesh:
    """An uploaded mesh (ufe_mesh_create). ``mesh`` is any object with the type_mesh
    attributes: base (V, nC, edge_index) and the AaAc arrays."""

    def __init__(self, mesh):
        L = nat.load()
        self.nV, self.nAc, self.nVAaAc = mesh.base.nV, mesh.nAc, mesh.nVAaAc
        d, keep = _mesh_desc(mesh)
        h = ct.c_void_p()
        rc = L.ufe_mesh_create(ct.byref(d), ct.byref(h))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_mesh_create")
        self._h = h   # the library copied everything it needs from ``keep``

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return nat.load().ufe_mesh_stream(self._h) or 0

    def close(self):
        if getattr(self, "_h", None):
            nat.load().ufe_mesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------- SSA
    def _ssa_structs(self, fields: dict, warm: dict | None):
        return _ssa_structs(self.nV, self.nAc, self.nVAaAc, fields, warm)

    def ssa_buffers(self) -> dict:
        """Zeroed host arrays for solve_ssa(buffers=...) (see the module's ssa_buffers)."""
        return ssa_buffers(self.nV, self.nAc, self.nVAaAc)

    def solve_ssa(self, fields: dict, params: dict, warm: dict | None = None, check: bool = True,
                  buffers: dict | None = None):
        """solve_SSA. Returns (status, outputs, stats). Outputs hold the solution U_SSA, V_SSA,
        Ux_SSA_Ac, Uy_SSA_Ac, N_AaAc and Up_SSA_Ac, Uo_SSA_Ac, eta_AaAc, S_AaAc, tau_c_AaAc,
        phi_fric_AaAc. With ``buffers`` (see ssa_buffers) the warm start is read from those
        arrays and every result written into them in place, with no allocation; the returned
        outputs are the same arrays."""
        L = nat.load()
        if buffers is None:
            si, sio, io, keep = self._ssa_structs(fields, warm)
            out = {k: np.zeros(self.nAc) for k in ("Up_SSA_Ac", "Uo_SSA_Ac")}
            out.update({k: np.zeros(self.nVAaAc) for k in ("eta_AaAc", "S_AaAc", "tau_c_AaAc", "phi_fric_AaAc")})
        else:
            if warm is not None:
                raise ValueError("with buffers the warm start is the buffers' content")
            _check_buffers(buffers, self.nV, self.nAc, self.nVAaAc)
            si, keep = _ssa_in(fields)
            io = {k: buffers[k] for k in SSA_INOUT_FIELDS}
            out = {k: buffers[k] for k in SSA_OUT_FIELDS}
        sio = nat.SsaInout(*(io[k].ctypes.data for k in SSA_INOUT_FIELDS))
        so = nat.SsaOut(*(out[k].ctypes.data for k in SSA_OUT_FIELDS))
        ps, _z = _params_struct(params)
        st = nat.SsaStats()
        rc = L.ufe_ssa_solve(self._h, ct.byref(ps), ct.byref(si), ct.byref(sio), ct.byref(so), ct.byref(st))
        if check and rc < 0:
            raise nat.UfeError(rc, "ufe_ssa_solve")
        out.update(io)
        return rc, out, stats_dict(st)

    def ssa_upload(self, fields: dict, params: dict, warm: dict | None = None):
        L = nat.load()
        si, sio, io, keep = self._ssa_structs(fields, warm)
        ps, _z = _params_struct(params)
        rc = L.ufe_ssa_upload(self._h, ct.byref(ps), ct.byref(si), ct.byref(sio))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_ssa_upload")

    def ssa_run(self, params: dict, check: bool = True):
        L = nat.load()
        ps, _z = _params_struct(params)
        st = nat.SsaStats()
        rc = L.ufe_ssa_run(self._h, ct.byref(ps), ct.byref(st))
        if check and rc < 0:
            raise nat.UfeError(rc, "ufe_ssa_run")
        return rc, stats_dict(st)

    def ssa_download(self):
        L = nat.load()
        io, sio, so = _download_structs(self.nV, self.nAc, self.nVAaAc)
        rc = L.ufe_ssa_download(self._h, ct.byref(sio), ct.byref(so))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_ssa_download")
        return io

    def ssa_vjp(self, dJ: dict, params: dict, geom_mesh=None, tol: float = 0.0, max_sweeps: int = 0,
                omega: float = 0.0, check: bool = True, method: int = 0, restart: int = 0,
                sweeps_per_iteration: int = 0):
        """VJP of the last solve on this handle (ufe_ssa_vjp). ``dJ`` holds dJ/du as U_SSA,
        V_SSA (nV) and Ux_SSA_Ac, Uy_SSA_Ac (nAc). With ``geom_mesh`` (an AaAc mesh with the
        Aa and Ac derivative stencils) dJ/dHi on Aa is returned too. Returns (status,
        outputs, stats)."""
        L = nat.load()
        keep = [np.ascontiguousarray(dJ[k], dtype=np.float64) for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac")]
        vin = nat.VjpIn(*(a.ctypes.data for a in keep))
        out = {k: np.zeros(self.nVAaAc) for k in nat.VJP_OUT_FIELDS if k != "dJ_dHi"}
        geom = None
        if geom_mesh is not None:
            gm = geom_mesh
            ncm = gm.CAaAc.shape[1]
            if gm.base.C.shape != (self.nV, ncm) or np.shape(gm.Nx) != (self.nV, ncm + 1) or \
                    np.shape(gm.Nx_Ac) != (self.nAc, 4) or np.shape(gm.Aci) != (self.nAc, 4):
                raise ValueError("geom_mesh arrays do not match this mesh (C: (nV, nC_mem), Nx: (nV, nC_mem+1))")
            gk = dict(nC=_i32(gm.base.nC), C=_i32(gm.base.C), Nx=_f64(gm.Nx), Ny=_f64(gm.Ny), Aci=_i32(gm.Aci),
                      Nx_Ac=_f64(gm.Nx_Ac), Ny_Ac=_f64(gm.Ny_Ac))
            keep.append(gk)
            geom = nat.VjpGeom(*(_ptr(gk[k]) for k in ("nC", "C", "Nx", "Ny", "Aci", "Nx_Ac", "Ny_Ac")))
            out["dJ_dHi"] = np.zeros(self.nV)
        vo = nat.VjpOut(*(_ptr(out.get(k)) for k in nat.VJP_OUT_FIELDS))
        vp = nat.VjpParams(tol, max_sweeps, omega, method, restart, sweeps_per_iteration)
        ps, _z = _params_struct(params)
        st = nat.VjpStats()
        rc = L.ufe_ssa_vjp(self._h, ct.byref(ps), ct.byref(vp), ct.byref(vin), ct.byref(geom) if geom else None,
                           ct.byref(vo), ct.byref(st))
        if check and rc < 0:
            raise nat.UfeError(rc, "ufe_ssa_vjp")
        return rc, out, dict(status=st.status, sweeps=st.sweeps, last_rel_update=st.last_rel_update,
                             device_ms=st.device_ms)

    def frictional_heating(self, mask_sheet):
        """bottom_frictional_heating from the last solve (ufe_ssa_frictional_heating)."""
        L = nat.load()
        m = np.ascontiguousarray(mask_sheet, dtype=np.int32)
        out = np.zeros(self.nV)
        rc = L.ufe_ssa_frictional_heating(self._h, m.ctypes.data, out.ctypes.data)
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_ssa_frictional_heating")
        return out

    # ---------------------------------------------------------------- geometry on the device
    def geometry_attach(self, mesh):
        """Upload the Aa and Ac derivative stencils of ``mesh`` (ufe_geometry_attach)."""
        L = nat.load()
        k = dict(nC=_i32(mesh.base.nC), C=_i32(mesh.base.C), Nx=_f64(mesh.Nx), Ny=_f64(mesh.Ny), Aci=_i32(mesh.Aci),
                 Nx_Ac=_f64(mesh.Nx_Ac), Ny_Ac=_f64(mesh.Ny_Ac), No_Ac=_f64(mesh.No_Ac), Np_Ac=_f64(mesh.Np_Ac))
        if k["C"].shape != (self.nV, mesh.CAaAc.shape[1]) or k["Nx"].shape != (self.nV, mesh.CAaAc.shape[1] + 1):
            raise ValueError("mesh stencils do not match this handle")
        g = nat.GeometryMesh(*(_ptr(k[n]) for n in nat.GEOM_MESH_FIELDS))
        rc = L.ufe_geometry_attach(self._h, ct.byref(g))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_geometry_attach")

    def geometry_update(self, Hi, Hb, SL) -> dict:
        """Derived geometry fields computed on the device (ufe_geometry_update)."""
        L = nat.load()
        ints = {"mask_ocean", "mask_ice", "mask_sheet", "mask_shelf", "mask_ocean_Ac", "mask_ice_Ac", "mask_sheet_Ac",
                "mask_shelf_Ac", "mask_gl_Ac"}
        out = {}
        for k in nat.GEOM_OUT_FIELDS:
            n = self.nAc if k.endswith("_Ac") else self.nV
            out[k] = np.zeros(n, dtype=np.int32 if k in ints else np.float64)
        go = nat.GeometryOut(*(out[k].ctypes.data for k in nat.GEOM_OUT_FIELDS))
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (Hi, Hb, SL)]
        rc = L.ufe_geometry_update(self._h, *(a.ctypes.data for a in arrs), ct.byref(go))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_geometry_update")
        return out

    def geometry_masks(self) -> dict:
        """Every mask of determine_masks from the last device geometry (ufe_geometry_masks):
        mask_<name> (nV) and mask_<name>_Ac (nAc) for each of nat.MASK_NAMES, plus the type
        masks mask (nV) and mask_Ac (nAc)."""
        L = nat.load()
        out = {k: np.zeros(self.nAc if k.endswith("_Ac") else self.nV, dtype=np.int32) for k in nat.MASK_OUT_FIELDS}
        mo = nat.MaskOut(*(out[k].ctypes.data for k in nat.MASK_OUT_FIELDS))
        rc = L.ufe_geometry_masks(self._h, ct.byref(mo))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_geometry_masks")
        return out

    def ssa_upload_geometry(self, Hi, Hb, SL, A_flow_mean, A_flow_mean_Ac, params: dict, beta=None,
                            warm: dict | None = None):
        """ufe_ssa_upload_geometry: the solve's inputs derived on the device from Hi, Hb, SL.
        A_flow_mean and A_flow_mean_Ac both None: the flow factors already on the device
        (ice_physical_properties)."""
        L = nat.load()
        _, sio, io, _ = self._ssa_structs({}, warm)
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
                for a in (Hi, Hb, SL, A_flow_mean, A_flow_mean_Ac)]
        b = None if beta is None else np.ascontiguousarray(beta, dtype=np.float64)
        ps, _z = _params_struct(params)
        rc = L.ufe_ssa_upload_geometry(self._h, ct.byref(ps), *(_ptr(a) for a in arrs), _ptr(b), ct.byref(sio))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_ssa_upload_geometry")

    def solve_sia_geometry(self, A_flow_Ac, params: dict):
        """ufe_sia_solve_geometry: the SIA on the device geometry of the last geometry update
        (A_flow_Ac None: the device's from ice_physical_properties)."""
        L = nat.load()
        nZ = len(params["zeta"])
        A = None if A_flow_Ac is None else np.asfortranarray(A_flow_Ac, dtype=np.float64)
        out = dict(D_SIA_3D_Ac=np.zeros((self.nAc, nZ), order="F"))
        for k in ("D_SIA_Ac", "Ux_SIA_Ac", "Uy_SIA_Ac", "Up_SIA_Ac", "Uo_SIA_Ac"):
            out[k] = np.zeros(self.nAc)
        for k in ("U_SIA", "V_SIA", "D_SIA"):
            out[k] = np.zeros(self.nV)
        so = nat.SiaOut(*(_ptr(out[k]) for k in ("D_SIA_3D_Ac", "D_SIA_Ac", "Ux_SIA_Ac", "Uy_SIA_Ac", "Up_SIA_Ac",
                                                  "Uo_SIA_Ac", "U_SIA", "V_SIA", "D_SIA")))
        ps, _z = _params_struct(params)
        rc = L.ufe_sia_solve_geometry(self._h, ct.byref(ps), _ptr(A), ct.byref(so))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_sia_solve_geometry")
        return out

    def solve_sia_3d(self, A_flow, dHb_dt, params: dict):
        """ufe_sia3d_solve: 3-D velocities on the device geometry (A_flow None: the device's
        from ice_physical_properties). Returns (U_3D, V_3D, W_3D)."""
        L = nat.load()
        nZ = len(params["zeta"])
        A = None if A_flow is None else np.asfortranarray(A_flow, dtype=np.float64)
        d = np.ascontiguousarray(dHb_dt, dtype=np.float64)
        outs = [np.zeros((self.nV, nZ), order="F") for _ in range(3)]
        so = nat.Sia3dOut(*(o.ctypes.data for o in outs))
        ps, _z = _params_struct(params)
        rc = L.ufe_sia3d_solve(self._h, ct.byref(ps), _ptr(A), d.ctypes.data, ct.byref(so))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_sia3d_solve")
        return tuple(outs)

    def ice_physical_properties(self, params: dict, Ti=None, flow_law: int = nat.UFE_FLOW_ARRHENIUS,
                                time: float = 0.0) -> dict:
        """ufe_ice_physical_properties on the device geometry of the last geometry update. Returns
        the fields the law writes: A_flow, Ti_pmp, Cpi, Ki (nV, nZ), A_flow_mean (nV), A_flow_Ac,
        Ti_Ac (nAc, nZ), A_flow_mean_Ac (nAc)."""
        L = nat.load()
        nZ = len(params["zeta"])
        shapes = dict(A_flow=(self.nV, nZ), Ti_pmp=(self.nV, nZ), Cpi=(self.nV, nZ), Ki=(self.nV, nZ),
                      A_flow_mean=(self.nV,), A_flow_Ac=(self.nAc, nZ), Ti_Ac=(self.nAc, nZ),
                      A_flow_mean_Ac=(self.nAc,))
        keys = ["A_flow", "A_flow_mean", "A_flow_Ac", "A_flow_mean_Ac"]
        if flow_law != nat.UFE_FLOW_MISMIP_MOD:
            keys += ["Ti_pmp", "Cpi", "Ki"]
        if flow_law == nat.UFE_FLOW_ARRHENIUS:
            keys.append("Ti_Ac")
        out = {k: np.zeros(shapes[k], order="F") for k in keys}
        po = nat.PhyspropOut(*(_ptr(out.get(k)) for k in nat.PHYSPROP_OUT_FIELDS))
        T = None if Ti is None else np.asfortranarray(Ti, dtype=np.float64)
        if T is not None and T.shape != (self.nV, nZ):
            raise ValueError("Ti must be (nV, nZ)")
        ps, _z = _params_struct(params)
        rc = L.ufe_ice_physical_properties(self._h, ct.byref(ps), int(flow_law), float(time), _ptr(T), ct.byref(po))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_ice_physical_properties")
        return out

    def triangles_attach(self, base, R, NxTri, NyTri):
        """Upload the triangle data of the upwind derivatives (ufe_triangles_attach): the base
        mesh's V, niTri, iTri, Tri, and mesh%R, NxTri, NyTri."""
        L = nat.load()
        k = dict(V=_f64(base.V), R=_f64(R), niTri=_i32(base.niTri), iTri=_i32(base.iTri), Tri=_i32(base.Tri),
                 NxTri=_f64(NxTri), NyTri=_f64(NyTri))
        nTri = k["Tri"].shape[0]
        if k["V"].shape != (self.nV, 2) or k["R"].shape != (self.nV,) or k["NxTri"].shape != (nTri, 3) or \
                k["NyTri"].shape != (nTri, 3) or k["Tri"].shape != (nTri, 3):
            raise ValueError("triangle arrays do not match this mesh")
        t = nat.TriangleMesh(nTri, *(_ptr(k[n]) for n in ("V", "R", "niTri", "iTri", "Tri", "NxTri", "NyTri")))
        rc = L.ufe_triangles_attach(self._h, ct.byref(t))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_triangles_attach")

    def upwind_derivatives_3d(self, params: dict, U_3D=None, V_3D=None, d=None):
        """ufe_upwind_derivatives_3d. U_3D, V_3D None: the device's last 3-D SIA velocities; d
        None: the device's Ti. Returns (ddx, ddy, pairs without an upwind triangle)."""
        L = nat.load()
        nZ = len(params["zeta"])
        arrs = [None if a is None else np.asfortranarray(a, dtype=np.float64) for a in (U_3D, V_3D, d)]
        for a in arrs:
            if a is not None and a.shape != (self.nV, nZ):
                raise ValueError("fields must be (nV, nZ)")
        ddx = np.zeros((self.nV, nZ), order="F")
        ddy = np.zeros((self.nV, nZ), order="F")
        miss = ct.c_int64(0)
        ps, _z = _params_struct(params)
        rc = L.ufe_upwind_derivatives_3d(self._h, ct.byref(ps), *(_ptr(a) for a in arrs), ddx.ctypes.data,
                                         ddy.ctypes.data, ct.byref(miss))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_upwind_derivatives_3d")
        return ddx, ddy, int(miss.value)

    def thickness_update(self, Hi, A, Cw, SMB_year, BMB, dt, Up_SIA_Ac=None, Up_SSA_Ac=None, mask_noice=None,
                         zero_edges=True):
        """calculate_ice_thickness_change on the device (ufe_thickness_update). Velocities left
        as None come from the handle's last SSA / SIA solves. Returns (Hi_new, Hi_prev,
        dHi_dt, dVi_in)."""
        L = nat.load()
        keep = dict(A=_f64(A), Cw=_f64(Cw), SMB=_f64(SMB_year), BMB=_f64(BMB),
                    usia=None if Up_SIA_Ac is None else _f64(Up_SIA_Ac),
                    ussa=None if Up_SSA_Ac is None else _f64(Up_SSA_Ac),
                    noice=None if mask_noice is None else _i32(mask_noice))
        ti = nat.ThicknessIn(_ptr(keep["A"]), _ptr(keep["Cw"]), _ptr(keep["usia"]), _ptr(keep["ussa"]),
                             _ptr(keep["SMB"]), _ptr(keep["BMB"]), _ptr(keep["noice"]), float(dt),
                             1 if zero_edges else 0)
        H = np.array(Hi, dtype=np.float64, copy=True)
        out = dict(Hi_prev=np.zeros(self.nV), dHi_dt=np.zeros(self.nV),
                   dVi_in=np.zeros(keep["Cw"].shape, order="F"))
        to = nat.ThicknessOut(*(out[k].ctypes.data for k in ("Hi_prev", "dHi_dt", "dVi_in")))
        rc = L.ufe_thickness_update(self._h, ct.byref(ti), H.ctypes.data, ct.byref(to))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_thickness_update")
        return H, out["Hi_prev"], out["dHi_dt"], out["dVi_in"]

    # ---------------------------------------------------------------- SIA
    def solve_sia(self, fields: dict, params: dict, want_3d: bool = True):
        L = nat.load()
        nZ = len(params["zeta"])
        keep = dict(mask_sheet_Ac=np.ascontiguousarray(fields["mask_sheet_Ac"], dtype=np.int32))
        for k in ("Hi_Ac", "dHs_dx_Ac", "dHs_dy_Ac", "dHs_dp_Ac", "dHs_do_Ac"):
            keep[k] = np.ascontiguousarray(fields[k], dtype=np.float64)
        keep["A_flow_Ac"] = np.asfortranarray(fields["A_flow_Ac"], dtype=np.float64)
        si = nat.SiaIn(*(keep[k].ctypes.data for k in ("mask_sheet_Ac", "Hi_Ac", "dHs_dx_Ac", "dHs_dy_Ac",
                                                        "dHs_dp_Ac", "dHs_do_Ac", "A_flow_Ac")))
        out = dict(D_SIA_3D_Ac=np.zeros((self.nAc, nZ), order="F") if want_3d else None)
        for k in ("D_SIA_Ac", "Ux_SIA_Ac", "Uy_SIA_Ac", "Up_SIA_Ac", "Uo_SIA_Ac"):
            out[k] = np.zeros(self.nAc)
        for k in ("U_SIA", "V_SIA", "D_SIA"):
            out[k] = np.zeros(self.nV)
        so = nat.SiaOut(*(_ptr(out[k]) for k in ("D_SIA_3D_Ac", "D_SIA_Ac", "Ux_SIA_Ac", "Uy_SIA_Ac", "Up_SIA_Ac",
                                                  "Uo_SIA_Ac", "U_SIA", "V_SIA", "D_SIA")))
        ps, _z = _params_struct(params)
        rc = L.ufe_sia_solve(self._h, ct.byref(ps), ct.byref(si), ct.byref(so))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_sia_solve")
        return out


def stats_dict(st) -> dict:
    n = min(64, st.linear_solves)
    return dict(status=st.status, picard_iterations=st.picard_iterations, linear_solves=st.linear_solves,
                resets=st.resets, not_converged=st.not_converged, total_sweeps=st.total_sweeps,
                last_RN=st.last_RN, last_max_residual=st.last_max_residual, sweeps=list(st.sweeps)[:n],
                device_ms=st.device_ms)


class Batch:
    """A batched ensemble (ufe_batch_create): independent SSA solves on meshes of uneven
    size, solved together in one persistent launch (replayed as a CUDA graph)."""

    def __init__(self, meshes, team_ctas: int = 0, rows_per_cta: int = 0, block: int = 0, use_graph: bool = True):
        L = nat.load()
        n = len(meshes)
        descs = (nat.MeshDesc * n)()
        keep = []
        self.sizes = []
        for i, m in enumerate(meshes):
            d, k = _mesh_desc(m)
            descs[i] = d
            keep.append(k)
            self.sizes.append((m.base.nV, m.nAc, m.nVAaAc))
        cfg = nat.BatchConfig(team_ctas, rows_per_cta, block, 1 if use_graph else 0)
        h = ct.c_void_p()
        rc = L.ufe_batch_create(descs, n, ct.byref(cfg), ct.byref(h))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_batch_create")
        self._h = h
        self.n = n

    def upload(self, i: int, fields: dict, params: dict, warm: dict | None = None, buffers: dict | None = None):
        """Member i's inputs; the warm start from ``warm`` or, in place, from ``buffers``
        (see ssa_buffers)."""
        L = nat.load()
        if buffers is None:
            si, sio, io, keep = _ssa_structs(*self.sizes[i], fields, warm)
        else:
            if warm is not None:
                raise ValueError("with buffers the warm start is the buffers' content")
            _check_buffers(buffers, *self.sizes[i])
            si, keep = _ssa_in(fields)
            sio, _ = _buffer_structs(buffers)
        ps, _z = _params_struct(params)
        rc = L.ufe_batch_upload(self._h, i, ct.byref(ps), ct.byref(si), ct.byref(sio))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_batch_upload")

    def run(self, params: dict, check: bool = True):
        """Solve every member. Returns (status, [stats per member], timing dict)."""
        L = nat.load()
        ps, _z = _params_struct(params)
        st = (nat.SsaStats * self.n)()
        member_ms = np.zeros(self.n)
        tm = nat.BatchTiming()
        tm.member_ms = member_ms.ctypes.data
        rc = L.ufe_batch_run(self._h, ct.byref(ps), st, ct.byref(tm))
        if check and rc < 0:
            raise nat.UfeError(rc, "ufe_batch_run")
        timing = {k: getattr(tm, k) for k, _ in nat.BatchTiming._fields_ if k != "member_ms"}
        timing["member_ms"] = member_ms
        return rc, [stats_dict(s) for s in st], timing

    def download(self, i: int, buffers: dict | None = None) -> dict:
        """Member i's results, into new arrays or in place into ``buffers``."""
        L = nat.load()
        if buffers is None:
            io, sio, so = _download_structs(*self.sizes[i])
        else:
            _check_buffers(buffers, *self.sizes[i])
            io = buffers
            sio, so = _buffer_structs(buffers)
        rc = L.ufe_batch_download(self._h, i, ct.byref(sio), ct.byref(so))
        if rc != nat.UFE_OK:
            raise nat.UfeError(rc, "ufe_batch_download")
        return io

    def close(self):
        if getattr(self, "_h", None):
            nat.load().ufe_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_plan(rows, resident_ctas: int, team_ctas: int = 0, rows_per_cta: int = 0, block: int = 0):
    """The ensemble planner (ufe_batch_plan, host only): (team size per member, classes as
    [(team size, teams)], grid CTAs)."""
    L = nat.load()
    r = np.ascontiguousarray(rows, dtype=np.int32)
    t = np.zeros(r.size, dtype=np.int32)
    cfg = nat.BatchConfig(team_ctas, rows_per_cta, block, 1)
    pl = nat.BatchPlan()
    rc = L.ufe_batch_plan(r.ctypes.data_as(ct.POINTER(ct.c_int32)), r.size, ct.byref(cfg), resident_ctas,
                          t.ctypes.data_as(ct.POINTER(ct.c_int32)), ct.byref(pl))
    if rc != nat.UFE_OK:
        raise nat.UfeError(rc, "ufe_batch_plan")
    classes = [(pl.class_team_ctas[c], pl.class_teams[c]) for c in range(pl.n_classes)]
    return t, classes, pl.grid_ctas


def batch_autotune(members, params: dict):
    """ufe_batch_autotune over (base, mesh, ssa_fields) members. Returns (best config dict,
    list of tried candidates)."""
    L = nat.load()
    n = len(members)
    descs = (nat.MeshDesc * n)()
    ins = (nat.SsaIn * n)()
    ios = (nat.SsaInout * n)()
    keep = []
    for i, (base, mesh, fields) in enumerate(members):
        d, k = _mesh_desc(mesh)
        si, sio, io, kk = _ssa_structs(base.nV, mesh.nAc, mesh.nVAaAc, fields, None)
        descs[i], ins[i], ios[i] = d, si, sio
        keep += [k, kk, io]
    ps, _z = _params_struct(params)
    best = nat.BatchConfig()
    log = (nat.BatchTuneEntry * 32)()
    cnt = ct.c_int32(0)
    rc = L.ufe_batch_autotune(n, descs, ct.byref(ps), ins, ios, ct.byref(best), log, 32, ct.byref(cnt))
    if rc != nat.UFE_OK:
        raise nat.UfeError(rc, "ufe_batch_autotune")
    tried = [{f: getattr(log[i], f) for f, _ in nat.BatchTuneEntry._fields_} for i in range(min(cnt.value, 32))]
    return {f: getattr(best, f) for f, _ in nat.BatchConfig._fields_}, tried
