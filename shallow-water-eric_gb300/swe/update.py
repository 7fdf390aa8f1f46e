"""Host-side mirror of the reference's ``MODULE update`` / ``MODULE fct``
interface (SOURCES/update.f90:1-16, SOURCES/fct.f90:1-5) over the C ABI.

    upd = Update(mesh, bath, params)        # construct_matrices
    dij, dt = upd.compute_dij(un)           # compute_dij + COMPUTE_DT
    unext = upd.euler(un)                   # euler(un, unext), inputs%dt = params.dt
    lij = upd.fct_positivity(hs, fctmat)    # FCT_positivity
    upd.lumped, upd.diag, upd.mass          # public module data

States are (syst_size, np) arrays in the reference numbering (Fortran
``un(S, np)`` layout).  Where the reference STOPs, a ``SweError`` is raised
with the C ABI's status code.  The device-resident fast path is
``upload`` / ``rk3_steps`` / ``download``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import lib as _L
from .cases import Params


def to_c_params(p: Params) -> _L.swe_params:
    return _L.swe_params(*p.fields())


class Update:
    def __init__(self, mesh=None, bath=None, params: Params | None = None, *, batch=None):
        """One mesh (``mesh``, ``bath``, ``params``) or a batch given as a list
        of ``(mesh, bath, params)`` tuples."""
        L = _L.load()
        self._L = L
        items = batch if batch is not None else [(mesh, bath, params)]
        self.n_inst = len(items)
        self.params = [p for _, _, p in items]
        self.np_ = np.array([m["rr"].shape[1] for m, _, _ in items], np.int32)
        me = np.array([m["jj"].shape[1] for m, _, _ in items], np.int32)
        self._me = me
        jj = np.concatenate([np.asfortranarray(m["jj"], np.int32).ravel(order="F") for m, _, _ in items])
        rr = np.concatenate([np.asfortranarray(m["rr"], np.float64).ravel(order="F") for m, _, _ in items])
        bb = np.concatenate([np.ascontiguousarray(b, np.float64) for _, b, _ in items])
        cp = (_L.swe_params * self.n_inst)(*[to_c_params(p) for p in self.params])
        self.S = self.params[0].syst_size
        h = ctypes.c_void_p()
        rc = L.swe_create_batch(ctypes.byref(h), self.n_inst, _L.ip(self.np_), _L.ip(me), _L.ip(jj), _L.dp(rr),
                                _L.dp(bb), cp)
        self.h = h
        if rc:
            msg = L.swe_last_error(h).decode() if h else ""
            if h:
                L.swe_destroy(h)
                self.h = None
            raise _L.SweError(rc, msg)
        self.node_off = np.concatenate([[0], np.cumsum(self.np_)]).astype(np.int64)

    def close(self):
        if getattr(self, "h", None):
            self._L.swe_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc:
            raise _L.SweError(rc, self._L.swe_last_error(self.h).decode())

    # ---- module data -------------------------------------------------------
    def sizes(self, inst=0):
        n = ctypes.c_int(); z = ctypes.c_int()
        self._check(self._L.swe_sizes(self.h, inst, ctypes.byref(n), ctypes.byref(z)))
        return n.value, z.value

    def matrices(self, inst=0):
        n, z = self.sizes(inst)
        ia = np.zeros(n + 1, np.int32); ja = np.zeros(z, np.int32)
        mass = np.zeros(z); lumped = np.zeros(n); diag = np.zeros(n, np.int32)
        cx = np.zeros(z); cy = np.zeros(z)
        self._check(self._L.swe_get_matrices(self.h, inst, _L.ip(ia), _L.ip(ja), _L.dp(mass), _L.dp(lumped),
                                             _L.ip(diag), _L.dp(cx), _L.dp(cy)))
        return dict(ia=ia, ja=ja, mass=mass, lumped=lumped, diag=diag, cx=cx, cy=cy)

    @property
    def lumped(self):
        return self.matrices()["lumped"]

    @property
    def diag(self):
        return self.matrices()["diag"]

    @property
    def mass(self):
        return self.matrices()["mass"]

    # ---- parameters / boundary data ---------------------------------------
    def set_params(self, p: Params, inst=0):
        self.params[inst] = p
        cp = to_c_params(p)
        self._check(self._L.swe_set_params(self.h, inst, ctypes.byref(cp)))

    def set_bath(self, bath, inst=0):
        b = np.ascontiguousarray(bath, np.float64)
        self._check(self._L.swe_set_bath(self.h, inst, _L.dp(b)))

    def set_dirichlet(self, comp, js, vals=None, inst=0):
        js = np.ascontiguousarray(js, np.int32)
        v = None if vals is None else np.ascontiguousarray(vals, np.float64)
        self._check(self._L.swe_set_dirichlet(self.h, inst, comp, len(js), _L.ip(js), _L.dp(v)))

    def set_dirichlet_anal(self, comp, js, inst=0):
        """Dirichlet data sol_anal(comp+1, rr(js), t) evaluated on the device
        at every stage's bdy time (type_test 5 and 13, components 0-2)."""
        js = np.ascontiguousarray(js, np.int32)
        self._check(self._L.swe_set_dirichlet_anal(self.h, inst, comp, len(js), _L.ip(js)))

    # ---- per-call operators (reference-shaped) ----------------------------
    def compute_dij(self, un, inst=0):
        u = np.asfortranarray(un, np.float64)
        n, z = self.sizes(inst)
        dij = np.zeros(z); dt = ctypes.c_double()
        self._check(self._L.swe_compute_dij(self.h, inst, _L.dp(u), _L.dp(dij), ctypes.byref(dt)))
        return dij, dt.value

    def euler(self, un, inst=0):
        u = np.asfortranarray(un, np.float64)
        out = np.zeros_like(u, order="F")
        self._check(self._L.swe_euler(self.h, inst, _L.dp(u), _L.dp(out)))
        return out

    def euler_intermediates(self, inst=0):
        n, z = self.sizes(inst)
        a = dict(dij_low=np.zeros(z), muij_low=np.zeros(z), alpha=np.zeros(n),
                 u_low=np.zeros((self.S, n), order="F"), res=np.zeros(n), fctmat=np.zeros(z),
                 rminus=np.zeros(n), lij=np.zeros(z))
        self._check(self._L.swe_euler_intermediates(self.h, inst, *[_L.dp(a[k]) for k in
                                                                  ("dij_low", "muij_low", "alpha", "u_low", "res",
                                                                   "fctmat", "rminus", "lij")]))
        return a

    def fct_positivity(self, unext_scaled, fctmat, inst=0):
        u = np.ascontiguousarray(unext_scaled, np.float64)
        f = np.ascontiguousarray(fctmat, np.float64)
        lij = np.zeros(len(f))
        self._check(self._L.swe_fct_positivity(self.h, inst, _L.dp(u), _L.dp(f), _L.dp(lij)))
        return lij

    def fct_generic(self, unext, maxn, minn, fctmat, dg=None, inst=0):
        """FCT_generic (SOURCES/SAFE/fct.f90:3-43): returns the limited copy of
        unext; dg defaults to the lumped mass."""
        u = np.array(unext, np.float64)
        a = [np.ascontiguousarray(x, np.float64) for x in (maxn, minn, fctmat)]
        d = None if dg is None else np.ascontiguousarray(dg, np.float64)
        self._check(self._L.swe_fct_generic(self.h, inst, _L.dp(u), _L.dp(a[0]), _L.dp(a[1]), _L.dp(a[2]),
                                            None if d is None else _L.dp(d)))
        return u

    # ---- diagnostics on the device-resident state ---------------------------
    def gauss_points(self, inst=0):
        """(rj (3 me,), rr_gauss (2, 3 me)) of the 3-point rule."""
        me = int(self._me[inst])
        rj = np.zeros(3 * me); rg = np.zeros(6 * me)
        self._check(self._L.swe_gauss_points(self.h, inst, _L.dp(rj), _L.dp(rg)))
        return rj, rg.reshape(-1, 2).T.copy()

    def norms(self, field=0, f_anal=None, inst=0):
        """(L1, L2) quadrature norms of field - f_anal on the device state
        (ns_anal_l1 / ns_anal_0); field may be lib.FIELD_H32."""
        fa = None if f_anal is None else np.ascontiguousarray(f_anal, np.float64)
        l1 = ctypes.c_double(); l2 = ctypes.c_double()
        self._check(self._L.swe_norms(self.h, inst, field, None if fa is None else _L.dp(fa),
                                      ctypes.byref(l1), ctypes.byref(l2)))
        return l1.value, l2.value

    # ---- movie frames (main.f90:119-143) -------------------------------------
    def frame_fields(self, hmax0, inst=0):
        """(hpz, h) of a movie frame from the device state: h + bath and h,
        with -1e-7 hmax0 + bath and 0 where h <= 1e-4 hmax0."""
        n = int(self.node_off[inst + 1] - self.node_off[inst])
        hpz = np.zeros(n); h = np.zeros(n)
        self._check(self._L.swe_frame_fields(self.h, inst, float(hmax0), _L.dp(hpz), _L.dp(h)))
        return hpz, h

    def frame_async(self, hpz_path, h_path, hmax0, inst=0):
        """Queue a movie frame: its fields are computed and copied on the
        GPU now and written as VTK files by a worker thread (hpz_k.vtk,
        h_k.vtk of the reference's time loop)."""
        self._check(self._L.swe_frame_async(self.h, inst, float(hmax0), str(hpz_path).encode(),
                                            str(h_path).encode()))

    def frames_wait(self):
        self._check(self._L.swe_frames_wait(self.h))

    # ---- gauges (main.f90:102-117) -------------------------------------------
    def set_gauges(self, rr, inst=None):
        """Point gauges at rr (2, n) (instances inst, default 0); returns their
        1-based elements.  Every later time step records (time, h, h + bath)
        interpolated at each gauge on the device."""
        pts = np.asfortranarray(np.asarray(rr, np.float64).reshape(2, -1))
        n = pts.shape[1]
        gi = np.zeros(n, np.int32) if inst is None else np.ascontiguousarray(inst, np.int32)
        elems = np.zeros(n, np.int32)
        self._check(self._L.swe_gauges_set(self.h, n, _L.ip(gi), _L.dp(pts.ravel(order="F")), _L.ip(elems)))
        self._n_gauges = n
        return elems

    def read_gauges(self, max_rows=4096):
        """Rows recorded since the last read: (times (rows, n), h (rows, n),
        h + bath (rows, n), lost)."""
        n = getattr(self, "_n_gauges", 0)
        out = np.zeros(3 * max(n, 1) * max_rows)
        rows = ctypes.c_int(); lost = ctypes.c_longlong()
        self._check(self._L.swe_gauges_read(self.h, max_rows, _L.dp(out), ctypes.byref(rows), ctypes.byref(lost)))
        a = out[:3 * n * rows.value].reshape(rows.value, n, 3)
        return a[:, :, 0], a[:, :, 1], a[:, :, 2], lost.value

    # ---- device-resident time loop ----------------------------------------
    def upload(self, un):
        """un: (S, sum np) concatenation of the instances' states, or a list."""
        if isinstance(un, (list, tuple)):
            un = np.hstack([np.asarray(x) for x in un])
        u = np.asfortranarray(un, np.float64)
        self._check(self._L.swe_upload(self.h, _L.dp(u)))

    def download(self):
        out = np.zeros((self.S, int(self.node_off[-1])), order="F")
        self._check(self._L.swe_download(self.h, _L.dp(out)))
        return out

    def download_split(self):
        u = self.download()
        return [u[:, self.node_off[b]:self.node_off[b + 1]] for b in range(self.n_inst)]

    def upload_ptr(self, host_ptr: int):
        """Upload from a raw host pointer (e.g. pinned memory) in the reference layout."""
        self._check(self._L.swe_upload(self.h, ctypes.cast(host_ptr, ctypes.POINTER(ctypes.c_double))))

    def download_ptr(self, host_ptr: int):
        self._check(self._L.swe_download(self.h, ctypes.cast(host_ptr, ctypes.POINTER(ctypes.c_double))))

    def upload_device(self, ptr: int):
        self._check(self._L.swe_upload_device(self.h, ctypes.c_void_p(ptr)))

    def download_device(self, ptr: int):
        self._check(self._L.swe_download_device(self.h, ctypes.c_void_p(ptr)))

    def set_time(self, time=0.0, t_final=1e300):
        t = np.broadcast_to(np.asarray(time, np.float64), (self.n_inst,)).copy()
        tf = np.broadcast_to(np.asarray(t_final, np.float64), (self.n_inst,)).copy()
        self._check(self._L.swe_set_time(self.h, _L.dp(t), _L.dp(tf)))

    def get_time(self):
        """(time, t_final, dt) per instance."""
        t = np.zeros(self.n_inst); tf = np.zeros(self.n_inst); dt = np.zeros(self.n_inst)
        self._check(self._L.swe_get_time(self.h, _L.dp(t), _L.dp(tf), _L.dp(dt)))
        return t, tf, dt

    def save_checkpoint(self, path):
        """The state and the instances' clocks as raw FP64 (npz), with the
        launch configuration: resuming from it continues the run bit for bit
        (the mixed state's double-float depth and FP32 momenta round-trip
        exactly through FP64, and every launch variant gives the same bits;
        the stored configuration keeps the resumed run's launch shapes)."""
        t, tf, dt = self.get_time()
        tuning = self.tuning
        spec = tuning.split("autotuned ", 1)[1] if "autotuned " in tuning else (
            tuning.split("fixed ", 1)[1] if "fixed " in tuning else "")
        np.savez(path, un=self.download(), time=t, t_final=tf, dt=dt, np_=self.np_, me=self._me,
                 S=self.S, precision=self.params[0].precision, tuning=np.array(spec))

    def load_checkpoint(self, path):
        with np.load(path) as z:
            if not (np.array_equal(z["np_"], self.np_) and np.array_equal(z["me"], self._me) and int(z["S"]) == self.S
                    and int(z["precision"]) == self.params[0].precision):
                raise ValueError("checkpoint of another mesh, system or precision")
            self.upload(z["un"])
            self.set_time(z["time"], z["t_final"])
            spec = str(z["tuning"]) if "tuning" in z.files else ""
        if spec:
            self.set_tuning(spec)

    def set_tuning(self, spec):
        """Launch exactly the variants of a tuning description (the text
        after "autotuned " in `tuning`) without timing."""
        self._check(self._L.swe_set_tuning(self.h, spec.encode()))

    def rk3_steps(self, nsteps):
        t = np.zeros(self.n_inst); dt = np.zeros(self.n_inst); n = ctypes.c_int()
        self._check(self._L.swe_rk3_steps(self.h, nsteps, _L.dp(t), _L.dp(dt), ctypes.byref(n)))
        return t, dt, n.value

    def rk3_steps_host_ptr(self, in_ptr, out_ptr, nsteps):
        """Upload from host pointer in_ptr (reference layout; 0 keeps the device
        state), nsteps steps, download to out_ptr (0 skips it): one call, one
        synchronisation."""
        t = np.zeros(self.n_inst); dt = np.zeros(self.n_inst); n = ctypes.c_int()
        cast = lambda p: ctypes.cast(p, ctypes.POINTER(ctypes.c_double)) if p else None
        self._check(self._L.swe_rk3_steps_host(self.h, cast(in_ptr), cast(out_ptr), nsteps, _L.dp(t), _L.dp(dt),
                                               ctypes.byref(n)))
        return t, dt, n.value

    def rk3_steps_host(self, un, nsteps):
        """rk3_steps_host_ptr on numpy arrays: returns the new state (S, np)."""
        u = np.asfortranarray(np.asarray(un, dtype=np.float64))
        if u.shape != (self.S, int(self.node_off[-1])):
            raise ValueError(f"state of shape {u.shape}, expected {(self.S, int(self.node_off[-1]))}")
        out = np.zeros_like(u, order="F")
        self.rk3_steps_host_ptr(u.ctypes.data, out.ctypes.data, nsteps)
        return out

    def total_mass(self):
        m = np.zeros(self.n_inst)
        self._check(self._L.swe_mass(self.h, _L.dp(m)))
        return m

    @property
    def last_launch_count(self):
        return int(self._L.swe_last_launch_count(self.h))

    @property
    def last_device_ms(self):
        return float(self._L.swe_last_device_ms(self.h))

    def profile_kernels(self, nsteps):
        """Average device ms per launch of each kernel kind (dt, node, low,
        fct, update) over nsteps event-bracketed steps."""
        out = np.zeros(len(_L.KERNEL_KINDS))
        self._check(self._L.swe_profile_kernels(self.h, nsteps, _L.dp(out)))
        return dict(zip(_L.KERNEL_KINDS, out.tolist()))

    def autotune(self):
        self._check(self._L.swe_autotune(self.h))
        return self.tuning

    @property
    def tuning(self):
        return self._L.swe_tuning(self.h).decode()


def from_case(case, precision=None, per_call=False):
    """Build an Update for a cases.Case (bath, params and Dirichlet data).
    Dirichlet values that change with time run in the device loop when the
    case lists them as analytic (``dirichlet_anal``: the device evaluates
    sol_anal at every stage's bdy time); otherwise the case needs
    ``per_call=True`` and a host loop that calls euler and bdy per stage."""
    anal = getattr(case, "dirichlet_anal", None) or []
    if not getattr(case, "bdy_fixed", True) and not per_call and not anal:
        raise ValueError(f"case {case.name}: Dirichlet values change with time; build it with per_call=True "
                         "and run it through the per-call operators")
    p = case.params
    if precision is not None:
        from dataclasses import replace
        p = replace(p, precision=precision)
    upd = Update(case.mesh, case.bath, p)
    for comp, js, vals in case.dirichlet:
        upd.set_dirichlet(comp, js, vals)
    if not per_call:
        for comp, js in anal:
            upd.set_dirichlet_anal(comp, js)
    return upd


def write_vtk_2d(path, jj, rr, field, title=None):
    """vtk_2d (SFEMaNS/FEMSUB/sub_plot.f90:1036-1095): one P1 scalar field as
    legacy-VTK text, byte for byte the reference's.  jj (3, me) 1-based,
    rr (2, np); title defaults to the file's name."""
    from pathlib import Path
    L = _L.load()
    jj = np.asfortranarray(jj, np.int32)
    rr = np.asfortranarray(rr, np.float64)
    f = np.ascontiguousarray(field, np.float64)
    if rr.shape[1] != f.size or jj.shape[0] != 3:
        raise ValueError("rr (2, np), jj (3, me) and a field of np values are required")
    rc = L.swe_write_vtk_2d(str(path).encode(), (title or Path(path).name).encode(), rr.shape[1], jj.shape[1],
                            _L.ip(jj.ravel(order="F")), _L.dp(rr.ravel(order="F")), _L.dp(f))
    if rc:
        raise _L.SweError(rc, f"cannot write {path}")
