"""Python handle over the C-ABI device solver (``dgadv_*`` in ``include/dgadv.h``)."""
import ctypes

import numpy as np

from . import _lib as L


class DeviceSolver:
    """One mesh + one configuration on one GPU.

    Arrays use the reference's shapes: ``cDisc`` K x N, ``u1Disc``/``u2Disc`` K x N,
    ``vNormalOnQuadEdge`` K x 3 x R.
    """

    def __init__(self, coordV, V0T, p, ordRK, precision='fp64', isSlopeLim=False,
                 typeSlopeLim='linear', idE0T=None, markE0TbdrD=None, markE0TbdrN=None,
                 device=0, flags=0, instances=None):
        """One mesh (coordV, V0T, markers), or an ensemble: ``instances`` a list of dicts with
        keys coordV, V0T and optionally idE0T, markE0TbdrD, markE0TbdrN (coordV / V0T ignored);
        the handle's arrays are then the instances' arrays stacked in order."""
        self._lib = L.load()
        self._h = None
        self.p = p
        self.N = (p + 1) * (p + 2) // 2
        self._keep = []
        meshes = instances if instances is not None else [dict(coordV=coordV, V0T=V0T, idE0T=idE0T,
                                                                markE0TbdrD=markE0TbdrD,
                                                                markE0TbdrN=markE0TbdrN)]
        arr = (L.Mesh * len(meshes))()
        self.instK = []
        for m, mesh in zip(meshes, arr):
            cv = L.f64(m['coordV'])
            vt = np.require(np.asarray(m['V0T'], dtype=np.int32), requirements=['F', 'A'])
            self._keep += [cv, vt]
            mesh.numT = vt.shape[0]
            mesh.numV = cv.shape[0]
            mesh.coordV = L.ptr(cv)
            mesh.V0T = L.ptr(vt, L._i32p)
            self.instK.append(vt.shape[0])
            if m.get('idE0T') is not None:
                a = np.require(np.asarray(m['idE0T'], dtype=np.int32), requirements=['F', 'A']); self._keep.append(a)
                mesh.idE0T = L.ptr(a, L._i32p)
            for name in ('markE0TbdrD', 'markE0TbdrN'):
                if m.get(name) is not None:
                    a = np.require(np.asarray(m[name], dtype=np.uint8), requirements=['F', 'A']); self._keep.append(a)
                    setattr(mesh, name, L.ptr(a, L._u8p))
        self.K = int(sum(self.instK))
        self.instStart = np.concatenate([[0], np.cumsum(self.instK)]).astype(np.int64)
        prm = L.Params()
        prm.p = p; prm.ordRK = ordRK
        prm.precision = {'fp64': L.FP64, 'fp32': L.FP32, 'df32': L.DF32}[precision]
        self.limiter = typeSlopeLim if isSlopeLim else 'none'
        self.precision = precision
        prm.isSlopeLim = 1 if isSlopeLim else 0
        prm.typeSlopeLim = L.LIMITER_TYPES[typeSlopeLim]
        prm.device = device; prm.flags = flags
        h = ctypes.c_void_p()
        if instances is None:
            st = self._lib.dgadv_create(arr, ctypes.byref(prm), ctypes.byref(h))
        else:
            st = self._lib.dgadv_create_ensemble(arr, len(meshes), ctypes.byref(prm), ctypes.byref(h))
        self._h = h.value
        if st != L.DGADV_OK:
            try:
                L.check(st, self._h)
            finally:
                self.close()

    def split(self, a):
        """Per-instance views of a stacked K x ... array."""
        return [a[self.instStart[i]:self.instStart[i + 1]] for i in range(len(self.instK))]

    # -------------------------------------------------------------------------------------
    def _c(self, st):
        L.check(st, self._h)

    def set_velocity(self, u1Disc, u2Disc, vNormalOnQuadEdge):
        u1, u2, vn = L.f64(u1Disc), L.f64(u2Disc), L.f64(vNormalOnQuadEdge)
        assert u1.shape == (self.K, self.N) and u2.shape == (self.K, self.N)
        assert vn.shape[:2] == (self.K, 3)
        self._c(self._lib.dgadv_set_velocity(self._h, L.ptr(u1), L.ptr(u2), L.ptr(vn)))

    def set_source_terms(self, timeFn, rhsTerms, cDV0T=None):
        n = len(timeFn)
        tf = np.asarray(timeFn, dtype=np.int32)
        if n == 0:
            self._c(self._lib.dgadv_set_source_terms(self._h, 0, None, None, None))
            return
        r = np.stack([L.f64(x) for x in rhsTerms], axis=2)       # K x N x n
        r = np.require(np.transpose(r, (0, 1, 2)), requirements=['F', 'A'])
        d = None
        if cDV0T is not None:
            d = np.require(np.stack([L.f64(x) for x in cDV0T], axis=2), requirements=['F', 'A'])
        self._c(self._lib.dgadv_set_source_terms(self._h, n, L.ptr(tf, L._i32p), L.ptr(r), L.ptr(d)))

    def set_state(self, cDisc):
        c = L.f64(cDisc)
        assert c.shape == (self.K, self.N)
        self._c(self._lib.dgadv_set_state(self._h, L.ptr(c)))

    def get_state(self, out=None):
        if out is None:
            out = np.zeros((self.K, self.N), order='F')
        self._c(self._lib.dgadv_get_state(self._h, L.ptr(out)))
        return out

    def limit_state(self, t):
        self._c(self._lib.dgadv_limit_state(self._h, float(t)))

    # ---- set-up on the device (functions of the built-in test cases) ----------------------
    def project_state(self, fns, t=0.0, qOrd=1):
        """projectFuncCont2DataDisc of f(t, x) into the state; fns: one (kind, params) pair or
        one per instance."""
        arr, keep = L.functions(_fn_list(fns))
        self._c(self._lib.dgadv_project_state(self._h, arr, len(arr), float(t), int(qOrd)))

    def set_velocity_function(self, fns):
        """Velocity data of u(x) computed on the device (replaces set_velocity's host arrays)."""
        arr, keep = L.functions(_fn_list(fns))
        self._c(self._lib.dgadv_set_velocity_function(self._h, arr, len(arr)))

    def l2_error(self, fns, t=0.0, qOrd=1):
        """computeL2Error of the state against f(t, x): a float, or one per instance when one
        function per instance is given."""
        specs = _fn_list(fns)
        arr, keep = L.functions(specs)
        out = np.zeros(len(specs))
        self._c(self._lib.dgadv_l2_error(self._h, arr, len(arr), float(t), int(qOrd), L.ptr(out)))
        return float(out[0]) if len(specs) == 1 else out

    # ---- transported species (transport problem) ------------------------------------------
    def transport_init(self, hDisc, cH0, maskTol=1e-6, isMask=True):
        """hDisc K x N depth; cH0 K x N x nSpecies (c h at t = 0)."""
        hd = L.f64(hDisc)
        c = L.f64(cH0)
        assert hd.shape == (self.K, self.N) and c.shape[:2] == (self.K, self.N)
        self.nSpecies = c.shape[2]
        self._c(self._lib.dgadv_transport_init(self._h, self.nSpecies, L.ptr(hd), L.ptr(c), float(maskTol),
                                               1 if isMask else 0))

    def transport_step(self, nSteps, nStep0, tau):
        self._c(self._lib.dgadv_transport_step(self._h, int(nSteps), int(nStep0), float(tau)))

    def transport_get(self, species):
        """(c h, c, mask) of one species."""
        cH = np.zeros((self.K, self.N), order='F')
        conc = np.zeros((self.K, self.N), order='F')
        mask = np.zeros(self.K, dtype=np.uint8)
        self._c(self._lib.dgadv_transport_get(self._h, int(species), L.ptr(cH), L.ptr(conc), L.ptr(mask, L._u8p)))
        return cH, conc, mask.astype(bool)

    # ---- implicit time stepping (handles created with flags=FLAG_IMPLICIT) -----------------
    def step_implicit(self, nSteps, nStep0, tau, ordRK, tol=1e-12, maxIter=2000, restart=50):
        """DIRK steps nStep0+1 .. nStep0+nSteps (GMRES per stage); returns (iterations, largest
        final relative residual)."""
        kr = L.Krylov(float(tol), int(maxIter), int(restart))
        it, rr = ctypes.c_int32(), ctypes.c_double()
        self._c(self._lib.dgadv_step_implicit(self._h, int(nSteps), int(nStep0), float(tau), int(ordRK),
                                              ctypes.byref(kr), ctypes.byref(it), ctypes.byref(rr)))
        return it.value, rr.value

    def solve_stationary(self, tol=1e-12, maxIter=2000, restart=50):
        """A c = sysV(0) from the current state; returns (iterations, final relative residual)."""
        kr = L.Krylov(float(tol), int(maxIter), int(restart))
        it, rr = ctypes.c_int32(), ctypes.c_double()
        self._c(self._lib.dgadv_solve_stationary(self._h, ctypes.byref(kr), ctypes.byref(it), ctypes.byref(rr)))
        return it.value, rr.value

    def get_lagrange(self):
        """projectDataDisc2DataLagr of the current state on the device: K x numP nodal values."""
        numP = 1 if self.p == 0 else (3 if self.p == 1 else 6)
        out = np.zeros((self.K, numP), order='F')
        n = ctypes.c_int32()
        self._c(self._lib.dgadv_get_lagrange(self._h, L.ptr(out), ctypes.byref(n)))
        assert n.value == numP
        return out

    def output(self, fileName, tLvl, types='vtk', varName='u_h'):
        """visualizeDataLagr(g, projectDataDisc2DataLagr(cDisc), varName, fileName, tLvl, types),
        enqueued: the files are written by the library's writer thread while later steps run."""
        self._c(self._lib.dgadv_output(self._h, varName.encode(), fileName.encode(), int(tLvl),
                                       L.output_types(types)))

    def output_wait(self):
        """Waits for every output file; raises if one could not be written."""
        self._c(self._lib.dgadv_output_wait(self._h))

    def step(self, nSteps, nStep0, tau):
        self._c(self._lib.dgadv_step(self._h, int(nSteps), int(nStep0), float(tau)))

    def sync(self):
        self._c(self._lib.dgadv_sync(self._h))

    def time_steps(self, nSteps, nStep0, tau):
        """Device time (ms) of nSteps, from CUDA events on the library's stream."""
        ms = ctypes.c_double()
        self._c(self._lib.dgadv_time_steps(self._h, int(nSteps), int(nStep0), float(tau), ctypes.byref(ms)))
        return ms.value

    def profile_kernels(self, nSteps, nStep0, tau):
        """Mean device ms per launch and launch counts of the kernel kinds
        (stage operator, time-derivative limiter, solution limiter)."""
        ms = np.zeros(4)
        n = np.zeros(4, dtype=np.int32)
        self._c(self._lib.dgadv_profile_kernels(self._h, int(nSteps), int(nStep0), float(tau),
                                                L.ptr(ms), L.ptr(n, L._i32p)))
        return ms[:3], n[:3]

    def set_option(self, option, value):
        self._c(self._lib.dgadv_set_option(self._h, int(option), int(value)))

    def get_option(self, option):
        v = ctypes.c_int32()
        self._c(self._lib.dgadv_get_option(self._h, int(option), ctypes.byref(v)))
        return v.value

    def link(self, other):
        """Steps `other` together with this handle from now on (dgadv_link); None unlinks all."""
        self._c(self._lib.dgadv_link(self._h, other._h if other is not None else None))

    def kernels_per_step(self):
        n = ctypes.c_int32()
        self._c(self._lib.dgadv_kernels_per_step(self._h, ctypes.byref(n)))
        return n.value

    # ---- discrete adjoint -------------------------------------------------------------------
    def set_velocity_modes(self, u1Modes, u2Modes, vNModes):
        """Velocity modes u_m: u1Modes, u2Modes K x N x M, vNModes K x 3 x R x M."""
        u1, u2, vn = L.f64(u1Modes), L.f64(u2Modes), L.f64(vNModes)
        M = u1.shape[-1]
        assert u1.shape == (self.K, self.N, M) and u2.shape == u1.shape and vn.shape[:2] == (self.K, 3)
        self.nModes = M
        self._c(self._lib.dgadv_set_velocity_modes(self._h, M, L.ptr(u1), L.ptr(u2), L.ptr(vn)))

    def set_velocity_theta(self, theta):
        th = L.f64(theta)
        self._c(self._lib.dgadv_set_velocity_theta(self._h, L.ptr(th)))

    def forward_record(self, nSteps, tau, nSnapshots=0):
        self._c(self._lib.dgadv_forward_record(self._h, int(nSteps), float(tau), int(nSnapshots)))

    def backward(self, dJdcT, want_theta=True):
        """(dJ/dc0 K x N, dJ/dtheta) for the last recorded run."""
        g = L.f64(dJdcT)
        assert g.shape == (self.K, self.N)
        g0 = np.zeros((self.K, self.N), order='F')
        gt = np.zeros(getattr(self, 'nModes', 0)) if want_theta else None
        self._c(self._lib.dgadv_backward(self._h, L.ptr(g), L.ptr(g0),
                                         L.ptr(gt) if gt is not None and gt.size else None))
        return g0, gt

    def close(self):
        if self._h:
            self._lib.dgadv_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _fn_list(fns):
    """A (kind, params) pair or a list of them."""
    if isinstance(fns, tuple) and len(fns) == 2 and not isinstance(fns[0], tuple):
        return [fns]
    return list(fns)
