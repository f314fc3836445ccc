"""Python mirror of the reference's ``NBody::KDTree`` interface over libnbkdt.

The method names follow ``src/KDTree/KDTree.h`` (pelahi/NBodylib) so tests read like the
reference's call sites. Arrays are numpy (host) or, when ``device=True``, torch CUDA
tensors whose storage is passed to the library as device pointers. Neighbour lists hold
tree indices (``KDTree.h:295``); ``GetPerm()[t]`` is the input index ("ID") of tree index
``t``; per-particle results are returned in input order.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi

TPHYS, TPROJ, TVEL, TPHS, TMETRIC = 0, 1, 2, 3, 4
KSPH, KGAUSS, KEPAN, KTH = 0, 1, 2, 3
FINDNEAREST, FINDNEARESTPOS, FINDNEARESTVEL, FINDNEARESTPHASE = 0, 1, 2, 3
PERIODIC_REF, PERIODIC_MIN_IMAGE = 0, 1
FOF3D, FOFVEL, FOF6D = 0, 1, 2
DEVICE_PTRS = 1


# device copies of periods, by (values, device): a tree built from device arrays passes its
# period as a device pointer, and a new 24-byte host-to-device copy per tree (blocking the
# host) would cost more than the call's own set-up
_DEVICE_PERIODS: dict = {}


def _device_period(torch, period, device):
    vals = tuple(float(x) for x in np.broadcast_to(np.asarray(period, np.float64), (3,)))
    key = (vals, str(device))
    t = _DEVICE_PERIODS.get(key)
    if t is None:
        if len(_DEVICE_PERIODS) > 64:
            _DEVICE_PERIODS.clear()
        t = torch.tensor(vals, dtype=torch.float64, device=device)
        _DEVICE_PERIODS[key] = t
    return t


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(ctypes.c_void_p)
    return ctypes.c_void_p(a.data_ptr())  # torch tensor


class KDTree:
    """GPU kd-tree with the reference constructor's arguments (KDTree.h:229-245)."""

    def __init__(self, pos, vel=None, mass=None, bucket_size=16, treetype=TPHYS,
                 kerntype=KEPAN, kernres=1000, splitting_criterion=0, aniso=0, scale_space=0,
                 period=None, device=False, stream=None):
        self._lib = _capi.load()
        self.device = device
        self._ball_cap = 0  # largest ball-search output so far (sizes the next buffer)
        if device:
            import torch
            self._torch = torch
            pos = pos.contiguous()
            self.n = pos.shape[0]
            per = None if period is None else _device_period(torch, period, pos.device)
            args = [pos, None if vel is None else vel.contiguous(),
                    None if mass is None else mass.contiguous()]
        else:
            pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
            self.n = pos.shape[0]
            vel = None if vel is None else np.ascontiguousarray(vel, np.float64).reshape(-1, 3)
            mass = None if mass is None else np.ascontiguousarray(mass, np.float64).reshape(-1)
            per = None if period is None else np.ascontiguousarray(
                np.broadcast_to(np.asarray(period, np.float64), (3,)))
            args = [pos, vel, mass]
        self._keep = (args, per)
        self.treetype = treetype
        self.nd = 6 if treetype == TPHS else 3
        self.periodic = period is not None
        self.bucket_size = bucket_size
        self.kernres = max(100, kernres)
        h = ctypes.c_void_p()
        _capi.check(self._lib.nbk_create(_ptr(args[0]), _ptr(args[1]), _ptr(args[2]), self.n,
                                         bucket_size, treetype, kerntype, kernres,
                                         splitting_criterion, aniso, scale_space, _ptr(per),
                                         DEVICE_PTRS if device else 0, ctypes.byref(h)))
        self._h = h
        if stream is not None:
            self.set_stream(stream)

    # ---- lifetime
    def close(self):
        if getattr(self, "_h", None):
            self._lib.nbk_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream):
        ptr = stream.cuda_stream if hasattr(stream, "cuda_stream") else stream
        _capi.check(self._lib.nbk_set_stream(self._h, ctypes.c_void_p(ptr)))

    def sync(self):
        _capi.check(self._lib.nbk_sync(self._h))

    # ---- allocation helpers
    def _empty(self, shape, dtype):
        if self.device:
            t = {np.int32: self._torch.int32, np.float64: self._torch.float64,
                 np.int64: self._torch.int64}[dtype]
            return self._torch.empty(shape, dtype=t, device="cuda")
        return np.empty(shape, dtype)

    # ---- getters (KDTree.h:282-289)
    def _counts(self):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        d = ctypes.c_int32()
        _capi.check(self._lib.nbk_get_counts(self._h, ctypes.byref(a), ctypes.byref(b),
                                             ctypes.byref(c), ctypes.byref(d)))
        return a.value, b.value, c.value, d.value

    def GetNumNodes(self):
        return self._counts()[1]

    def GetNumLeafNodes(self):
        return self._counts()[2]

    def GetBucketSize(self):
        return self._counts()[3]

    def GetPerm(self):
        out = self._empty(self.n, np.int32)
        _capi.check(self._lib.nbk_get_perm(self._h, _ptr(out)))
        return out

    def GetKernel(self):
        t = np.empty(self.kernres)
        kn = ctypes.c_double()
        _capi.check(self._lib.nbk_get_kernel(self._h, _ptr(t), ctypes.byref(kn)))
        return t, kn.value

    # ---- kNN (KDTree.h:300-313)
    def FindNearest(self, k, periodic_mode=PERIODIC_REF):
        """All-particle FindNearest(tt): (nn[n,k] tree indices, d2[n,k]), row = tree index."""
        nn = self._empty((self.n, k), np.int32)
        d2 = self._empty((self.n, k), np.float64)
        _capi.check(self._lib.nbk_knn(self._h, k, FINDNEAREST, periodic_mode, _ptr(nn), _ptr(d2)))
        return nn, d2

    def FindNearestPos(self, k, periodic_mode=PERIODIC_REF):
        nn = self._empty((self.n, k), np.int32)
        d2 = self._empty((self.n, k), np.float64)
        _capi.check(self._lib.nbk_knn(self._h, k, FINDNEARESTPOS, periodic_mode, _ptr(nn),
                                      _ptr(d2)))
        return nn, d2

    def FindNearestPosPoints(self, x, k, periodic_mode=PERIODIC_REF):
        """FindNearestPos(Double_t *x) for every row of x."""
        if not self.device:
            x = np.ascontiguousarray(x, np.float64).reshape(-1, 3)
        nq = x.shape[0]
        nn = self._empty((nq, k), np.int32)
        d2 = self._empty((nq, k), np.float64)
        _capi.check(self._lib.nbk_knn_points(self._h, _ptr(x), nq, k, periodic_mode, _ptr(nn),
                                             _ptr(d2)))
        return nn, d2

    def FindNearestPhase(self, k):
        """FindNearestPhase(tt) for every particle of a phase-space tree: the plain phase
        distance whatever the tree's aniso (KDFindNearest.cxx:347-361)."""
        nn = self._empty((self.n, k), np.int32)
        d2 = self._empty((self.n, k), np.float64)
        _capi.check(self._lib.nbk_knn(self._h, k, FINDNEARESTPHASE, PERIODIC_REF, _ptr(nn),
                                      _ptr(d2)))
        return nn, d2

    def FindNearestVel(self, k):
        """FindNearestVel(tt) for every particle of a velocity tree."""
        nn = self._empty((self.n, k), np.int32)
        d2 = self._empty((self.n, k), np.float64)
        _capi.check(self._lib.nbk_knn(self._h, k, FINDNEARESTVEL, PERIODIC_REF, _ptr(nn),
                                      _ptr(d2)))
        return nn, d2

    def FindNearestPhasePoints(self, x, k):
        """FindNearestPhase(Double_t *x, Double_t *v) for rows (x, y, z, vx, vy, vz)."""
        if not self.device:
            x = np.ascontiguousarray(x, np.float64).reshape(-1, 6)
        nq = x.shape[0]
        nn = self._empty((nq, k), np.int32)
        d2 = self._empty((nq, k), np.float64)
        _capi.check(self._lib.nbk_knn_phase_points(self._h, _ptr(x), nq, k, _ptr(nn), _ptr(d2)))
        return nn, d2

    def FindNearestTargets(self, targets, k, variant=FINDNEAREST, periodic_mode=PERIODIC_REF):
        """FindNearest(tt) / FindNearestPos(tt) for the given tree indices: row i belongs
        to targets[i]."""
        targets = self._targets(targets)
        nn = self._empty((len(targets), k), np.int32)
        d2 = self._empty((len(targets), k), np.float64)
        _capi.check(self._lib.nbk_knn_targets(self._h, _ptr(targets), len(targets), k, variant,
                                              periodic_mode, _ptr(nn), _ptr(d2)))
        return nn, d2

    def FindNearestPoints(self, x, k):
        """FindNearest(Double_t *x) for every row of x, in the tree's own space: 3 positions
        (physical tree), 3 velocities (velocity tree) or x, y, z, vx, vy, vz (phase space)."""
        if not self.device:
            x = np.ascontiguousarray(x, np.float64).reshape(-1, self.nd)
        nq = x.shape[0]
        nn = self._empty((nq, k), np.int32)
        d2 = self._empty((nq, k), np.float64)
        _capi.check(self._lib.nbk_knn_coords(self._h, _ptr(x), nq, k, _ptr(nn), _ptr(d2)))
        return nn, d2

    # ---- SPH (KDTree.h:407-425)
    def CalcDensity(self, k=64):
        rho = self._empty(self.n, np.float64)
        _capi.check(self._lib.nbk_density(self._h, k, _ptr(rho)))
        return rho

    def CalcVelDensity(self, nsmooth=64, nsearch=64):
        out = self._empty(self.n, np.float64)
        _capi.check(self._lib.nbk_veldensity(self._h, nsmooth, nsearch, _ptr(out)))
        return out

    def CalcDensityAndVelDensity(self, k=64, nsmooth=64):
        rho = self._empty(self.n, np.float64)
        vd = self._empty(self.n, np.float64)
        _capi.check(self._lib.nbk_density_veldensity(self._h, k, nsmooth, _ptr(rho), _ptr(vd)))
        return rho, vd

    def CalcDensityParticle(self, targets, k=64):
        targets = self._targets(targets)
        out = self._empty(len(targets), np.float64)
        _capi.check(self._lib.nbk_density_particles(self._h, _ptr(targets), len(targets), k,
                                                    _ptr(out)))
        return out

    def CalcVelDensityParticle(self, targets, nsmooth=64, nsearch=64):
        targets = self._targets(targets)
        out = self._empty(len(targets), np.float64)
        _capi.check(self._lib.nbk_veldensity_particles(self._h, _ptr(targets), len(targets),
                                                       nsmooth, nsearch, _ptr(out)))
        return out

    def CalcDensityPosition(self, x, k=64):
        """CalcDensityPosition at each row of x (n, 3), physical trees."""
        x = self._pts(x)
        out = self._empty(x.shape[0], np.float64)
        _capi.check(self._lib.nbk_density_points(self._h, _ptr(x), x.shape[0], k, _ptr(out)))
        return out

    def CalcVelDensityPosition(self, x, v, nsmooth=64, nsearch=64):
        """CalcVelDensityPosition at each row of x with the velocity in the same row of v."""
        x, v = self._pts(x), self._pts(v)
        out = self._empty(x.shape[0], np.float64)
        _capi.check(self._lib.nbk_veldensity_points(self._h, _ptr(x), _ptr(v), x.shape[0],
                                                    nsmooth, nsearch, _ptr(out)))
        return out

    # ---- SPH smoothing (KDCalcSmoothQuantities.cxx:393-766, 922-1091, 1209-1306,
    # 1539-1700). rho: densities in input order (the reference's densityset = 1, i.e. what
    # CalcDensity returned), or None to compute CalcDensity(Nsmooth) first. Targets are
    # tree indices, points an (nq, 3) array; matrices come back as (.., 3, 3).
    def _vec(self, a, shape):
        if a is None:
            return None
        if self.device:
            return a.to(self._torch.float64).contiguous()
        return np.ascontiguousarray(a, np.float64).reshape(shape)

    def _pts(self, x):
        if self.device:
            return x.to(self._torch.float64).contiguous()
        return np.ascontiguousarray(x, np.float64).reshape(-1, 3)

    def CalcSmoothVel(self, Nsmooth=64, rho=None):
        out = self._empty((self.n, 3), np.float64)
        _capi.check(self._lib.nbk_smooth_vel(self._h, Nsmooth, _ptr(self._vec(rho, (-1,))),
                                             _ptr(out)))
        return out

    def CalcSmoothVelDisp(self, smvel, Nsmooth=64, rho=None):
        out = self._empty((self.n, 3, 3), np.float64)
        _capi.check(self._lib.nbk_smooth_vel_disp(self._h, Nsmooth, _ptr(self._vec(rho, (-1,))),
                                                  _ptr(self._vec(smvel, (-1, 3))), _ptr(out)))
        return out

    def _moment(self, fn, smvel, smveldisp, Nsmooth, rho):
        out = self._empty((self.n, 3), np.float64)
        _capi.check(fn(self._h, Nsmooth, _ptr(self._vec(rho, (-1,))),
                       _ptr(self._vec(smvel, (-1, 3))), _ptr(self._vec(smveldisp, (-1, 9))),
                       _ptr(out)))
        return out

    def CalcSmoothVelSkew(self, smvel, smveldisp, Nsmooth=64, rho=None):
        return self._moment(self._lib.nbk_smooth_vel_skew, smvel, smveldisp, Nsmooth, rho)

    def CalcSmoothVelKurtosis(self, smvel, smveldisp, Nsmooth=64, rho=None):
        return self._moment(self._lib.nbk_smooth_vel_kurtosis, smvel, smveldisp, Nsmooth, rho)

    def CalcVelDensityWithPhysDensity(self, Nsmooth=64, Nsearch=64, rho=None):
        out = self._empty(self.n, np.float64)
        _capi.check(self._lib.nbk_veldensity_physdensity(self._h, Nsmooth, Nsearch,
                                                         _ptr(self._vec(rho, (-1,))), _ptr(out)))
        return out

    def CalcVelDensityWithPhysDensityParticle(self, targets, Nsmooth=64, Nsearch=64, rho=None):
        targets = self._targets(targets)
        out = self._empty(len(targets), np.float64)
        _capi.check(self._lib.nbk_veldensity_physdensity_particles(
            self._h, _ptr(targets), len(targets), Nsmooth, Nsearch, _ptr(self._vec(rho, (-1,))),
            _ptr(out)))
        return out

    def CalcSmoothVelParticle(self, targets, Nsmooth=64, rho=None):
        targets = self._targets(targets)
        out = self._empty((len(targets), 3), np.float64)
        _capi.check(self._lib.nbk_smooth_vel_particles(self._h, _ptr(targets), len(targets),
                                                       Nsmooth, _ptr(self._vec(rho, (-1,))),
                                                       _ptr(out)))
        return out

    def CalcSmoothVelPosition(self, x, Nsmooth=64, rho=None):
        x = self._pts(x)
        out = self._empty((x.shape[0], 3), np.float64)
        _capi.check(self._lib.nbk_smooth_vel_points(self._h, _ptr(x), x.shape[0], Nsmooth,
                                                    _ptr(self._vec(rho, (-1,))), _ptr(out)))
        return out

    def CalcSmoothVelDispParticle(self, targets, smvel, Nsmooth=64, rho=None):
        targets = self._targets(targets)
        out = self._empty((len(targets), 3, 3), np.float64)
        _capi.check(self._lib.nbk_smooth_vel_disp_particles(
            self._h, _ptr(targets), len(targets), Nsmooth, _ptr(self._vec(rho, (-1,))),
            _ptr(self._vec(smvel, (-1, 3))), _ptr(out)))
        return out

    def CalcSmoothVelDispPosition(self, x, smvel, Nsmooth=64, rho=None):
        x = self._pts(x)
        out = self._empty((x.shape[0], 3, 3), np.float64)
        _capi.check(self._lib.nbk_smooth_vel_disp_points(
            self._h, _ptr(x), x.shape[0], Nsmooth, _ptr(self._vec(rho, (-1,))),
            _ptr(self._vec(smvel, (-1, 3))), _ptr(out)))
        return out

    def CalcSmoothLocalMeanParticle(self, targets, weight, Nsmooth=64, rho=None):
        targets = self._targets(targets)
        out = self._empty(len(targets), np.float64)
        _capi.check(self._lib.nbk_smooth_local_mean_particles(
            self._h, _ptr(targets), len(targets), Nsmooth, _ptr(self._vec(rho, (-1,))),
            _ptr(self._vec(weight, (-1,))), _ptr(out)))
        return out

    def CalcSmoothLocalMeanPosition(self, x, weight, Nsmooth=64, rho=None):
        x = self._pts(x)
        out = self._empty(x.shape[0], np.float64)
        _capi.check(self._lib.nbk_smooth_local_mean_points(
            self._h, _ptr(x), x.shape[0], Nsmooth, _ptr(self._vec(rho, (-1,))),
            _ptr(self._vec(weight, (-1,))), _ptr(out)))
        return out

    def CalcSmoothLocalDispParticle(self, targets, weight, mean, Nsmooth=64, rho=None):
        targets = self._targets(targets)
        out = self._empty(len(targets), np.float64)
        _capi.check(self._lib.nbk_smooth_local_disp_particles(
            self._h, _ptr(targets), len(targets), Nsmooth, _ptr(self._vec(rho, (-1,))),
            _ptr(self._vec(weight, (-1,))), _ptr(self._vec(mean, (-1,))), _ptr(out)))
        return out

    def CalcSmoothLocalDispPosition(self, x, weight, mean, Nsmooth=64, rho=None):
        x = self._pts(x)
        out = self._empty(x.shape[0], np.float64)
        _capi.check(self._lib.nbk_smooth_local_disp_points(
            self._h, _ptr(x), x.shape[0], Nsmooth, _ptr(self._vec(rho, (-1,))),
            _ptr(self._vec(weight, (-1,))), _ptr(self._vec(mean, (-1,))), _ptr(out)))
        return out

    def _targets(self, targets):
        if self.device:
            return targets.to(self._torch.int32).contiguous()
        return np.ascontiguousarray(np.atleast_1d(targets), np.int32)

    # ---- ball search (KDTree.h:341-376)
    def SearchBallPosTagged(self, targets, fdist2):
        """Batch of SearchBallPosTagged(tt, fdist2): CSR (offsets[nt+1], tree indices)."""
        targets = self._targets(targets)
        return self._ball(self._lib.nbk_ball_tagged, targets, len(targets), fdist2)

    def SearchBallPosTaggedPoints(self, x, fdist2):
        if not self.device:
            x = np.ascontiguousarray(x, np.float64).reshape(-1, 3)
        return self._ball(self._lib.nbk_ball_tagged_points, x, x.shape[0], fdist2)

    def _ball(self, fn, q, nq, fdist2):
        """One call (count, scan, fill) when the output buffer sized by the largest result
        of an earlier call on this tree is large enough; otherwise a counting call first
        (the C ABI returns NBK_ERR_INVALID with *total set when out_capacity is short)."""
        offsets = self._empty(nq + 1, np.int64)
        total = ctypes.c_int64()
        cap = self._ball_cap
        out = None
        if cap > 0:
            out = self._empty(cap, np.int32)
        st = fn(self._h, _ptr(q), nq, float(fdist2), _ptr(offsets), _ptr(out), cap,
                ctypes.byref(total))
        if st == 0 and out is not None:
            return offsets, out[: total.value]
        if st not in (0, 1):
            _capi.check(st)
        cap = max(total.value, 1)
        out = self._empty(cap, np.int32)
        _capi.check(fn(self._h, _ptr(q), nq, float(fdist2), _ptr(offsets), _ptr(out), cap,
                       ctypes.byref(total)))
        self._ball_cap = max(self._ball_cap, cap)
        return offsets, out[: total.value]

    def SearchBallPos(self, target, fdist2, imark, nn, dist2):
        """SearchBallPos(tt, fdist2, imark, nn, dist2): marks input-order arrays in place."""
        _capi.check(self._lib.nbk_ball_mark(self._h, int(target), float(fdist2), int(imark),
                                            _ptr(nn), _ptr(dist2)))

    # ---- FOF (KDTree.h:480-503)
    def FOF(self, fdist, minnum=8, order=0):
        group = self._empty(self.n, np.int32)
        ng = ctypes.c_int32()
        _capi.check(self._lib.nbk_fof(self._h, float(fdist), int(minnum), int(order),
                                      _ptr(group), ctypes.byref(ng)))
        return group, ng.value

    def FOFCriterion(self, comparator, params, minnum=8, order=0):
        p = np.zeros(20)
        p[: len(params)] = params
        if self.device:
            p = self._torch.as_tensor(p, device="cuda")
        group = self._empty(self.n, np.int32)
        ng = ctypes.c_int32()
        _capi.check(self._lib.nbk_fof_criterion(self._h, int(comparator), _ptr(p), int(minnum),
                                                int(order), _ptr(group), ctypes.byref(ng)))
        return group, ng.value

    # ---- FOF over given neighbour lists (KDTree.h:497-515, KDFOF.cxx:380-640)
    def FOFNNCriterion(self, comparator, params, nn, minnum=8):
        """nn: (n, numNN) tree indices, rows by tree index (as FindNearest returns them).
        Returns (group[n] in input order, numbered by decreasing size, ngroup)."""
        return self._fof_nn(comparator, params, nn, None, None, minnum)

    def FOFNNDistCriterion(self, comparator, params, nn, values, pidx, minnum=8):
        """As FOFNNCriterion, with params[pidx[k]] replaced per particle by values (tree
        order): the values the reference takes from distfunc(numNN, dist2[t])."""
        return self._fof_nn(comparator, params, nn, values, pidx, minnum)

    def _fof_nn(self, comparator, params, nn, values, pidx, minnum):
        p = np.zeros(8)
        p[: min(8, len(params))] = np.asarray(params, np.float64)[:8]
        if self.device:
            p = self._torch.from_numpy(p).cuda()
            nn = nn.to(self._torch.int32).contiguous()
            vals = None if values is None else values.to(self._torch.float64).contiguous()
            pi = None if pidx is None else self._torch.as_tensor(
                np.asarray(pidx, np.int32)).cuda()
        else:
            nn = np.ascontiguousarray(nn, np.int32)
            vals = None if values is None else np.ascontiguousarray(values, np.float64)
            pi = None if pidx is None else np.ascontiguousarray(pidx, np.int32)
        numnn = nn.shape[1]
        group = self._empty(self.n, np.int32)
        ng = ctypes.c_int32()
        if vals is None:
            _capi.check(self._lib.nbk_fof_nn_criterion(self._h, int(comparator), _ptr(p), numnn,
                                                       _ptr(nn), int(minnum), _ptr(group),
                                                       ctypes.byref(ng)))
        else:
            _capi.check(self._lib.nbk_fof_nn_dist_criterion(
                self._h, int(comparator), _ptr(p), numnn, _ptr(nn), _ptr(vals), len(pi), _ptr(pi),
                int(minnum), _ptr(group), ctypes.byref(ng)))
        return group, ng.value

    # ---- adjoint (no reference counterpart)
    def DensityAdjoint(self, k, w):
        w = w if self.device else np.ascontiguousarray(w, np.float64)
        rho = self._empty(self.n, np.float64)
        gp = self._empty((self.n, 3), np.float64)
        gm = self._empty(self.n, np.float64)
        _capi.check(self._lib.nbk_density_adjoint(self._h, k, _ptr(w), _ptr(rho), _ptr(gp),
                                                  _ptr(gm)))
        return rho, gp, gm


class BatchedDensity:
    """Many independent per-group trees built and searched together (nbk_batch_*).

    pos: (N, 3), mass: (N,), offsets: (G+1,) CSR over groups (host arrays, or torch CUDA
    tensors with device=True). bucket_size <= 0 selects the autotuned leaf size.
    """

    def __init__(self, pos, mass, offsets, bucket_size=0, kerntype=KSPH, kernres=1000,
                 device=False):
        self._lib = _capi.load()
        self.device = device
        if device:
            import torch
            self._torch = torch
            args = (pos.contiguous(), None if mass is None else mass.contiguous(),
                    offsets.to(torch.int64).contiguous())
        else:
            args = (np.ascontiguousarray(pos, np.float64).reshape(-1, 3),
                    None if mass is None else np.ascontiguousarray(mass, np.float64),
                    np.ascontiguousarray(offsets, np.int64))
        self._keep = args
        self.n = int(args[2][-1])
        self.ngroups = len(args[2]) - 1
        h = ctypes.c_void_p()
        _capi.check(self._lib.nbk_batch_create(_ptr(args[0]), _ptr(args[1]), _ptr(args[2]),
                                               self.ngroups, bucket_size, kerntype, kernres,
                                               DEVICE_PTRS if device else 0, ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.nbk_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        b, q = ctypes.c_int32(), ctypes.c_int32()
        buf = ctypes.create_string_buffer(1 << 14)
        _capi.check(self._lib.nbk_batch_get_params(self._h, ctypes.byref(b), ctypes.byref(q),
                                                   buf, len(buf)))
        return b.value, q.value, buf.value.decode()

    def query_mapping(self):
        """1: a warp serves one query at a time; 0: a lane per query (32 per warp)."""
        w = ctypes.c_int32()
        _capi.check(self._lib.nbk_batch_get_query_mapping(self._h, ctypes.byref(w)))
        return w.value

    def set_query_mapping(self, warp_per_query):
        _capi.check(self._lib.nbk_batch_set_query_mapping(self._h, int(warp_per_query)))

    def _out(self):
        if self.device:
            return self._torch.empty(self.n, dtype=self._torch.float64, device="cuda")
        return np.empty(self.n)

    def density(self, k=32, use_graph=True, out=None):
        rho = self._out() if out is None else out
        _capi.check(self._lib.nbk_batch_density(self._h, k, _ptr(rho), 1 if use_graph else 0))
        return rho

    def density_pertree(self, k=32, out=None):
        rho = self._out() if out is None else out
        _capi.check(self._lib.nbk_batch_density_pertree(self._h, k, _ptr(rho)))
        return rho

    def density_pertree_search(self, k=32, out=None):
        """The per-group search loop over the already-built forest (no builds)."""
        rho = self._out() if out is None else out
        _capi.check(self._lib.nbk_batch_density_pertree_search(self._h, k, _ptr(rho)))
        return rho

    def set_stream(self, stream):
        """Run on a caller's CUDA stream (a torch Stream or a raw handle). Graph capture
        needs a stream other than the legacy default stream."""
        ptr = stream.cuda_stream if hasattr(stream, "cuda_stream") else stream
        _capi.check(self._lib.nbk_batch_set_stream(self._h, ctypes.c_void_p(ptr)))
