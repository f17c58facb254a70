"""Many geometries in one basis handle: batched Fock builds, RHF and gradients.

One ``BatchBasis`` holds every geometry's shells, shell pairs and work plan;
each Fock build is one CUDA-graph launch whose class kernels cover the
quartets of all geometries (quartets never couple two geometries).  Matrices
are packed: geometry g's n_g x n_g block starts at ``offsets[g]``.  The SCF
iterations run in FP64 on the GPU, batched over geometries of equal basis size
(the library's batched Jacobi eigensolver on stacks of Fock matrices), with
per-geometry DIIS.

The reference builds one molecule per process (src/bin/rchem.rs:10-90); this
is new capability, with the reference's energy conventions.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .basis import Basis, _after_torch, _check_f64, _same_kind
from .bse import expand_shells, load_bse


class BatchBasis(Basis):
    def __init__(self, geometries, basis_set_name="6-31g-fit"):
        """geometries: list of (atomnos, coords_bohr)."""
        doc = load_bse(basis_set_name)
        self.name = basis_set_name if isinstance(basis_set_name, str) else "custom"
        Zs, Rs, gnat = [], [], []
        atom, ls, nprim, exps, coefs = [], [], [], [], []
        a0 = 0
        for Z, R in geometries:
            Z = np.asarray(Z, dtype=np.int32).reshape(-1)
            R = np.asarray(R, dtype=np.float64).reshape(-1, 3)
            sh = expand_shells(Z, doc)
            atom.append(sh.atom + a0)
            ls.append(sh.l)
            nprim.append(sh.nprim)
            exps.append(sh.exps)
            coefs.append(sh.coefs)
            Zs.append(Z)
            Rs.append(R)
            gnat.append(len(Z))
            a0 += len(Z)
        self.atomnos = np.ascontiguousarray(np.concatenate(Zs), dtype=np.int32)
        self.coords = np.ascontiguousarray(np.concatenate(Rs), dtype=np.float64)
        self.geom_natoms = np.ascontiguousarray(gnat, dtype=np.int32)
        cat = lambda xs, dt: np.ascontiguousarray(np.concatenate(xs), dtype=dt)  # noqa: E731
        sa, sl, sn = cat(atom, np.int32), cat(ls, np.int32), cat(nprim, np.int32)
        se, sc = cat(exps, np.float64), cat(coefs, np.float64)
        h = C.c_void_p()
        L = _lib.lib()
        _lib.check(L.rchem_batch_create(C.byref(h), len(gnat), self.geom_natoms.ctypes.data, len(self.atomnos),
                                        self.atomnos.ctypes.data, self.coords.ctypes.data, len(sl), sa.ctypes.data,
                                        sl.ctypes.data, sn.ctypes.data, se.ctypes.data, sc.ctypes.data))
        self._h = h
        self.nbf = int(L.rchem_basis_nbf(h))
        self.ngeom = len(gnat)
        packed = C.c_longlong()
        self.geom_nbf = np.zeros(self.ngeom, dtype=np.int32)
        self.offsets = np.zeros(self.ngeom, dtype=np.int64)
        _lib.check(L.rchem_basis_layout(h, None, C.byref(packed), self.geom_nbf.ctypes.data,
                                        self.offsets.ctypes.data))
        self.packed = int(packed.value)
        self.atom0 = np.concatenate([[0], np.cumsum(self.geom_natoms)[:-1]]).astype(np.int64)

    def _new(self, like=None, shape=None):
        shape = shape or (self.packed,)
        if like is not None and hasattr(like, "is_cuda") and like.is_cuda:
            import torch

            return torch.empty(shape, dtype=torch.float64, device=like.device)
        return np.empty(shape, dtype=np.float64)

    def block(self, packed, g):
        n, o = int(self.geom_nbf[g]), int(self.offsets[g])
        return packed[o:o + n * n].reshape(n, n)


def _packed_matrix(fn, bb: BatchBasis):
    import torch

    out = torch.empty(bb.packed, dtype=torch.float64, device="cuda")
    _after_torch(bb, out)
    _lib.check(fn(bb.handle, C.c_void_p(out.data_ptr()), _lib.DEVICE))
    return out


def eigh(A):
    """Eigenvalues (ascending) and eigenvectors (columns) of a batch of small
    symmetric FP64 CUDA matrices (..., n, n), n <= 64, through
    rchem_eigh_batched (one thread block per matrix, cyclic Jacobi), queued on
    torch's current stream.  Reads the lower triangle, like torch.linalg.eigh."""
    import torch

    if not (A.is_cuda and A.dtype == torch.float64):
        raise ValueError("eigh takes CUDA float64 matrices")
    n = A.shape[-1]
    lead = A.shape[:-2]
    A = A.reshape(-1, n, n).contiguous()
    w = torch.empty(A.shape[:-1], dtype=torch.float64, device=A.device)
    V = torch.empty_like(A)
    _lib.check(_lib.lib().rchem_eigh_batched(n, A.shape[0], C.c_void_p(A.data_ptr()), C.c_void_p(w.data_ptr()),
                                             C.c_void_p(V.data_ptr()),
                                             C.c_void_p(torch.cuda.current_stream(A.device).cuda_stream)))
    return w.reshape(*lead, n), V.reshape(*lead, n, n)


def jk(bb: BatchBasis, D, J, K, schwarz_tau=1e-12, fp32_tau=0.0, emulated=False):
    """One Fock build over every geometry: packed device vectors D -> J, K."""
    if not _same_kind(D, J, K):
        raise ValueError("D, J and K must be CUDA tensors")
    for X, name in ((D, "D"), (J, "J"), (K, "K")):
        _check_f64(X, name, numel=bb.packed)
    o = _lib.JKOpts(schwarz_tau=schwarz_tau if schwarz_tau > 0 else -1.0, fp32_tau=fp32_tau, where=_lib.DEVICE,
                    emulated=1 if emulated else 0)
    _after_torch(bb, D, J, K)
    _lib.check(_lib.lib().rchem_jk_direct(bb.handle, C.c_void_p(D.data_ptr()), C.c_void_p(J.data_ptr()),
                                          C.c_void_p(K.data_ptr()), C.byref(o)))


def rhf_batch(bb: BatchBasis, thresh_e=1e-10, thresh_d=1e-7, max_iter=128, diis=8, fp32_tau=0.0,
              schwarz_tau=1e-12, emulated=False):
    """RHF for every geometry of ``bb`` at once; returns per-geometry energies,
    the packed D and W, iteration count and convergence flags.

    The iterations run on one side stream shared by torch and the library
    (the handle is moved to it), so no host synchronisation orders them; the
    caller's stream waits for the results."""
    import torch

    caller = torch.cuda.current_stream()
    side = torch.cuda.Stream()
    side.wait_stream(caller)
    bb.set_stream(side.cuda_stream)
    with torch.cuda.stream(side):
        res = _rhf_batch(bb, thresh_e, thresh_d, max_iter, diis, fp32_tau, schwarz_tau, emulated)
    caller.wait_stream(side)
    for key in ("D", "W"):  # allocated on the side stream, used on the caller's
        res[key].record_stream(caller)
    return res


def _rhf_batch(bb, thresh_e, thresh_d, max_iter, diis, fp32_tau, schwarz_tau, emulated):
    import torch

    dev = torch.device("cuda")
    L = _lib.lib()
    S = _packed_matrix(L.rchem_S, bb)
    H = _packed_matrix(L.rchem_T, bb) + _packed_matrix(L.rchem_V, bb)
    nocc = np.array([int(bb.atomnos[bb.atom0[g]:bb.atom0[g] + bb.geom_natoms[g]].sum()) // 2
                     for g in range(bb.ngeom)])
    # geometries grouped by basis size; gather/scatter indices into the packed vectors
    groups = []
    for n in sorted(set(bb.geom_nbf.tolist())):
        gs = np.nonzero(bb.geom_nbf == n)[0]
        idx = torch.as_tensor((bb.offsets[gs][:, None] + np.arange(n * n)[None, :]).reshape(-1), device=dev)
        occ = set(nocc[gs].tolist())
        if len(occ) != 1:
            raise ValueError("geometries of one basis size must have one electron count")
        groups.append((n, gs, idx, occ.pop()))

    def gather(v, grp):
        n, gs, idx, _ = grp
        return v[idx].view(len(gs), n, n)

    st = []
    for grp in groups:
        n, gs, idx, no = grp
        Sg = gather(S, grp)
        w, U = eigh(Sg)
        X = (U * w.rsqrt().unsqueeze(-2)) @ U.transpose(-1, -2)
        st.append({"X": X, "S": Sg, "H": gather(H, grp), "focks": [], "errs": []})

    def densities(Fs):
        D = torch.empty(bb.packed, dtype=torch.float64, device=dev)
        extra = []
        for grp, s_, F in zip(groups, st, Fs):
            n, gs, idx, no = grp
            X = s_["X"]
            eps, Cp = eigh(X.transpose(-1, -2) @ F @ X)
            Cm = X @ Cp
            Co = Cm[..., :no]
            D[idx] = (Co @ Co.transpose(-1, -2)).reshape(-1)
            extra.append((eps, Cm))
        return D, extra

    D, _ = densities([s_["H"] for s_ in st])
    J = torch.empty_like(D)
    K = torch.empty_like(D)
    e_old = None
    it = 0
    conv = np.zeros(bb.ngeom, dtype=bool)
    e_g = np.zeros(bb.ngeom)
    for it in range(1, max_iter + 1):
        jk(bb, D, J, K, schwarz_tau, fp32_tau, emulated)
        F = H + 2.0 * J - K
        Fx, egs = [], []
        for grp, s_ in zip(groups, st):
            n, gs, idx, no = grp
            Fg, Dg = gather(F, grp), gather(D, grp)
            egs.append(((s_["H"] + Fg) * Dg).sum(dim=(-1, -2)))
            X = s_["X"]
            err = X.transpose(-1, -2) @ (Fg @ Dg @ s_["S"] - s_["S"] @ Dg @ Fg) @ X
            s_["focks"].append(Fg)
            s_["errs"].append(err)
            if len(s_["focks"]) > diis:
                s_["focks"].pop(0)
                s_["errs"].pop(0)
            m = len(s_["focks"])
            if m >= 2 and diis > 0:
                E = torch.stack(s_["errs"], dim=1).reshape(len(gs), m, -1)
                Bm = torch.zeros((len(gs), m + 1, m + 1), dtype=torch.float64, device=dev)
                Bm[:, :m, :m] = E @ E.transpose(-1, -2)
                Bm[:, m, :m] = -1.0
                Bm[:, :m, m] = -1.0
                rhs = torch.zeros((len(gs), m + 1), dtype=torch.float64, device=dev)
                rhs[:, m] = -1.0
                # solve_ex: no host synchronisation; a singular system keeps that geometry's F
                c, info = torch.linalg.solve_ex(Bm, rhs)
                ext = torch.einsum("gk,gkij->gij", c[:, :m], torch.stack(s_["focks"], dim=1))
                Fx.append(torch.where((info != 0)[:, None, None], Fg, ext))
            else:
                Fx.append(Fg)
        D_old = D
        D, _ = densities(Fx)
        # one device-to-host transfer per iteration: every energy and max |dD|
        host = torch.cat(egs + [(D - D_old).abs().max().reshape(1)]).cpu().numpy()
        pos = 0
        for grp in groups:
            e_g[grp[1]] = host[pos:pos + len(grp[1])]
            pos += len(grp[1])
        dmax = float(host[-1])
        if e_old is not None:
            conv = np.abs(e_g - e_old) < thresh_e
            if conv.all() and dmax < thresh_d:
                e_old = e_g.copy()
                break
        e_old = e_g.copy()
    # final energies and W at the converged densities
    jk(bb, D, J, K, schwarz_tau, fp32_tau, emulated)
    F = H + 2.0 * J - K
    W = torch.empty_like(D)
    Dn = torch.empty_like(D)
    for grp, s_ in zip(groups, st):
        n, gs, idx, no = grp
        Fg = gather(F, grp)
        e_g[gs] = ((s_["H"] + Fg) * gather(D, grp)).sum(dim=(-1, -2)).cpu().numpy()
        X = s_["X"]
        eps, Cp = eigh(X.transpose(-1, -2) @ Fg @ X)
        Cm = X @ Cp
        Co = Cm[..., :no]
        W[idx] = ((Co * eps[..., :no].unsqueeze(-2)) @ Co.transpose(-1, -2)).reshape(-1)
        Dn[idx] = gather(D, grp).reshape(-1)
    from .scf import nuclear_repulsion

    e_nuc = np.array([nuclear_repulsion(bb.atomnos[bb.atom0[g]:bb.atom0[g] + bb.geom_natoms[g]],
                                        bb.coords[bb.atom0[g]:bb.atom0[g] + bb.geom_natoms[g]])
                      for g in range(bb.ngeom)])
    return {"e_elec": e_g.copy(), "e_nuc": e_nuc, "e_total": e_g + e_nuc, "D": Dn, "W": W, "iterations": it,
            "converged": bool(conv.all())}


def rhf_native(bb: Basis, thresh_e=1e-10, thresh_d=1e-7, max_iter=128, diis=8, fp32_tau=0.0, schwarz_tau=1e-12,
               emulated=False):
    """The same RHF as rhf_batch, run entirely inside librchem_gpu.so
    (rchem_rhf): one C call, every geometry's matrices on the GPU, Jacobi
    diagonalisation (each geometry n <= 64).  Works on a single-geometry Basis
    too.  Returns per-geometry energies and the packed D and W."""
    import torch

    ng = getattr(bb, "ngeom", 1)
    packed = getattr(bb, "packed", bb.nbf * bb.nbf)
    o = _lib.SCFOpts(thresh_e=thresh_e, thresh_d=thresh_d, max_iter=max_iter, diis=diis,
                     jk=_lib.JKOpts(schwarz_tau=schwarz_tau if schwarz_tau > 0 else -1.0, fp32_tau=fp32_tau,
                                    where=_lib.DEVICE, emulated=1 if emulated else 0))
    e_elec, e_nuc = np.zeros(ng), np.zeros(ng)
    D = torch.empty(packed, dtype=torch.float64, device="cuda")
    W = torch.empty_like(D)
    it, conv = C.c_int(0), C.c_int(0)
    _after_torch(bb, D, W)
    _lib.check(_lib.lib().rchem_rhf(bb.handle, C.byref(o), None, e_elec.ctypes.data, e_nuc.ctypes.data,
                                    C.c_void_p(D.data_ptr()), C.c_void_p(W.data_ptr()), C.byref(it), C.byref(conv)))
    return {"e_elec": e_elec, "e_nuc": e_nuc, "e_total": e_elec + e_nuc, "D": D, "W": W, "iterations": it.value,
            "converged": bool(conv.value)}


def gradient_batch(bb: BatchBasis, res: dict, schwarz_tau=1e-12, fp32_tau=0.0, emulated=False):
    """Nuclear gradients of every geometry: one set of adjoint-kernel launches
    (precision options as in scf.gradient); returns a list of (natoms_g x 3) arrays."""
    import torch

    if not _same_kind(res["D"], res["W"]):
        raise ValueError("D and W must be CUDA tensors")
    for key in ("D", "W"):
        _check_f64(res[key], key, numel=bb.packed)
    g = torch.empty(3 * len(bb.atomnos), dtype=torch.float64, device="cuda")
    o = _lib.JKOpts(schwarz_tau=schwarz_tau if schwarz_tau > 0 else -1.0, fp32_tau=fp32_tau, where=_lib.DEVICE,
                    emulated=1 if emulated else 0)
    _after_torch(bb, res["D"], res["W"], g)
    _lib.check(_lib.lib().rchem_gradient(bb.handle, C.c_void_p(res["D"].data_ptr()), C.c_void_p(res["W"].data_ptr()),
                                         C.c_void_p(g.data_ptr()), C.byref(o)))
    G = g.view(-1, 3).cpu().numpy()
    return [G[bb.atom0[k]:bb.atom0[k] + bb.geom_natoms[k]] for k in range(bb.ngeom)]
