"""Hamiltonian-vector products of the order-0 general-XRCC Hamiltonian of three fragments,
without forming H.

general-XRCC builds H one element at a time (build_H.py:38-188: monomer, dimer and trimer
elements, embedded into the product basis by general-XRCC/hamiltonian.py:18-80) and
diagonalises it densely.  For three fragments of 14 spatial orbitals with 40 states per
charge (+1, 0, -1) the product space has 120^3 = 1.7 M states and one trimer charge block
alone is 64 000 x 64 000 (33 GB in FP64), so here H is never formed.  w = H v is evaluated
term by term on a vector stored block by block over charge triples (c0, c1, c2), each block
a row-major (n_c0, n_c1, n_c2) array:

  monomers  w[i0,i1,i2] += H1_f[i_f, j_f] v[..., j_f, ...]          f = 0, 1, 2
  pairs     w += (H2_ab x 1_s) v                                       (a,b) = (0,1), (1,2), (0,2)
            H2_ab: the pair's dimer blocks (build_H.py:48-102) as dense per-total-charge
            sector matrices from XRDimerPlan; on (0,2) the spectator phase (-1)^(n_1 dq)
            of moving an odd number of operators past fragment 1's creation string
  triples   w[x,y,z] += a sum P[x,x',r,s] R2[y,y',r] R3[z,z',s] v[x',y',z']
            P = R1 . W (+ delta U / 4), the first stage of trimer.XRTrimerPlan, once per build

For a trimer charge block with fragment order (x, y, z) (build_H.py:103-188 case analysis,
the fragment carrying the two-index density first), the product runs in three GEMM stages
that never touch an n^3 x n^3 object:

  A  T1[x',y',z,s]  = sum_z'     v[x',y',z'] R3t[z,s,z']          (R3 transposed once per build)
  B  T2p[x,z,y',r]  = a sum_x',s T1[x',y',z,s] P[x',x,r,s]       (x' as K-concatenated segments;
                                                                    the GEMM's scatter epilogue
                                                                    writes the layout of stage C)
  C  w[x,z,y]      += sum_y',r   T2p[x,z,y',r] R2[y,y',r]

each one GEMM with K contiguous in both operands, about 2 n^4 N^2 FLOPs per block instead of
the 2 n^6 of a stored block.  Blocks of a fragment order other than (0, 1, 2) read a permuted
copy of v (order x, y, z) and add into a permuted accumulator (order x, z, y).

TrimerHvPlan is the plan as host data (GEMM task records over named flat buffers), so the
same plan drives the device (XRTrimerHamiltonian, grouped launches of libxrh's GEMM) and can
be executed by a NumPy interpreter in the tests.  Every GEMM record follows the
xrh_gemm_task / xrh_gemm_segment contract of include/xrh.h.
"""
import numpy as np
import torch

from . import _lib
from ._lib import call, ptr, stream_ptr
from .gemm import GroupedGemm
from .trimer import _case, _phase

IDENTITY = (0, 1, 2)
PAIRS = ((0, 1), (1, 2), (0, 2))         # the spectator of each pair: 2, 0, 1


def pair_sector_layout(chg_a, chg_b, ns_a, ns_b):
    """Sector layout of XRDimerPlan(layout='sector'): {total charge t: (base, dim)} with
    base[c_a] the first row of charge block (c_a, t - c_a), rows (i_a, i_b) row-major."""
    out = {}
    for ca in chg_a:
        for cb in chg_b:
            base, dim = out.get(ca + cb, ({}, 0))
            base[ca] = dim
            out[ca + cb] = (base, dim + ns_a[ca] * ns_b[cb])
    return out


def _seg(A, lda, B, ldb, K, alpha=1.0, flags=0, sA=0, sB=0):
    return dict(A=A, lda=lda, B=B, ldb=ldb, K=K, alpha=float(alpha), flags=flags, sA=sA, sB=sB)


def _task(M, N, C, ldc, segs, mode=1, batch=1, sC=0):
    return dict(M=M, N=N, C=C, ldc=ldc, segs=segs, mode=mode, batch=batch, sC=sC)


def _vname(order):
    return "v" if order == IDENTITY else "v%d%d%d" % order


def _wname(order):
    return "w" if order == IDENTITY else "w%d%d%d" % order


class TrimerHvPlan:
    """GEMM records of one three-fragment H x v (host data only).

    charges:     three charge lists (state order of each fragment: charge blocks in this order)
    n_states:    three {charge: number of states}
    n_elec:      three reference electron counts (charge c holds n_elec - c electrons)
    Ns:          spin orbitals per fragment
    avail:       avail(f, op, bra_chg, ket_chg) -> True when fragment f has that density block
    total_charge: None for the whole product space, or one total charge (H conserves it)
    monomer_scale: factor of the monomer tasks: 1 when the pair blocks are the dimer couplings
                 alone (XRDimerPlan output 'split'); -1 when they are the full pair
                 Hamiltonians H1 x 1 + 1 x H1 + H2 (output 'full'), which count every monomer
                 twice over the three pairs

    Buffers are named: 'v', 'w' (the vectors), 'vXYZ'/'wXYZ' (permuted copies for fragment
    order XYZ), 'Pt', 'R3t', 'T1', 'T2p' (intermediates, sizes in self.sizes) and external
    keys ('rho', f, op, bc, kc), ('H1', f, c), ('H2', pair, t), ('W', kind, order),
    ('Uq', order), ('eye', n).  A reference is (buffer, element offset)."""

    def __init__(self, charges, n_states, n_elec, Ns, avail, total_charge=None, monomer_scale=1.0):
        self.monomer_scale = float(monomer_scale)
        self.charges = [list(c) for c in charges]
        self.ns = [dict(n) for n in n_states]
        self.n_elec = list(n_elec)
        self.Ns = list(Ns)
        ns = self.ns
        triples = [(a, b, c) for a in self.charges[0] for b in self.charges[1] for c in self.charges[2]]
        if total_charge is not None:
            triples = [t for t in triples if sum(t) == total_charge]
        self.triples = triples
        self.off, self.shape = {}, {}
        dim = 0
        for t in triples:
            self.off[t] = dim
            self.shape[t] = tuple(ns[f][t[f]] for f in range(3))
            dim += int(np.prod(self.shape[t]))
        self.dim = dim
        self.sizes = {"v": dim, "w": dim}
        self.build_tasks, self.permutes, self.mid_permutes = [], [], []
        self.launches = [[], [], []]
        self.orders_v, self.orders_w = set(), set()
        self.pair_layout = [pair_sector_layout(self.charges[a], self.charges[b], ns[a], ns[b]) for a, b in PAIRS]
        self._monomers(avail)
        self._pairs()
        self._trimers(avail)
        for o in sorted(self.orders_v - {IDENTITY}):
            self.sizes[_vname(o)] = dim
        for o in sorted(self.orders_w - {IDENTITY}):
            self.sizes[_wname(o)] = dim
        self.flops_apply = sum(_task_flops(t) for L in self.launches for t in L)
        self.flops_build = sum(_task_flops(t) for t in self.build_tasks)

    # ---------------------------------------------------------------------------------
    def _alloc(self, name, n):
        o = self.sizes.get(name, 0)
        self.sizes[name] = o + int(n)
        return o

    def _monomers(self, avail):
        """H1_f on axis f of every block (build_H.py:38-47); fragment f has a monomer block
        for charge c when it has the rho^ca block (c, c)."""
        a = self.monomer_scale
        for t in self.triples:
            n0, n1, n2 = self.shape[t]
            o = self.off[t]
            if avail(0, "ca", t[0], t[0]):
                self.launches[0].append(_task(n0, n1 * n2, ("w", o), n1 * n2,
                                              [_seg((("H1", 0, t[0]), 0), n0, ("v", o), n1 * n2, n0, alpha=a,
                                                    flags=2)]))
            if avail(1, "ca", t[1], t[1]):
                self.launches[0].append(_task(n1, n2, ("w", o), n2,
                                              [_seg((("H1", 1, t[1]), 0), n1, ("v", o), n2, n1, alpha=a, flags=2,
                                                    sB=n1 * n2)],
                                              batch=n0, sC=n1 * n2))
            if avail(2, "ca", t[2], t[2]):
                self.launches[0].append(_task(n0 * n1, n2, ("w", o), n2,
                                              [_seg(("v", o), n2, (("H1", 2, t[2]), 0), n2, n2, alpha=a)]))

    def _pairs(self):
        """(H2_ab x 1_s) v for the three pairs, every source block in one task per output block."""
        in_layout = set(self.triples)
        for p, (a, b) in enumerate(PAIRS):
            s = 3 - a - b
            lay = self.pair_layout[p]
            for t in self.triples:
                tot = t[a] + t[b]
                base, dimt = lay[tot]
                segs = []
                for ca2 in self.charges[a]:
                    cb2 = tot - ca2
                    if cb2 not in self.charges[b] or abs(ca2 - t[a]) > 2:
                        continue
                    src = [0, 0, 0]
                    src[a], src[b], src[s] = ca2, cb2, t[s]
                    src = tuple(src)
                    if src not in in_layout:
                        continue
                    H = (("H2", p, tot), base[t[a]] * dimt + base[ca2])
                    na2, nb2 = self.ns[a][ca2], self.ns[b][cb2]
                    if (a, b) == (0, 1):
                        # v in fragment order (2, 0, 1): the block is [i2][(j0 j1)], K-contiguous
                        self.orders_v.add((2, 0, 1))
                        segs.append(_seg(H, dimt, ("v201", self.off[src]), na2 * nb2, na2 * nb2))
                    elif (a, b) == (1, 2):
                        segs.append(_seg(("v", self.off[src]), na2 * nb2, H, dimt, na2 * nb2))
                    else:
                        # spectator 1: (-1)^(n_1 dq), n_1 its electron-count parity, dq the parity of
                        # the charge moved between fragments 0 and 2
                        odd = (self.n_elec[1] - t[1]) % 2 == 1 and (t[0] - ca2) % 2 == 1
                        self.orders_v.add((1, 0, 2))
                        self.orders_w.add((1, 0, 2))
                        segs.append(_seg(("v102", self.off[src]), na2 * nb2, H, dimt, na2 * nb2,
                                         alpha=-1.0 if odd else 1.0))
                if not segs:
                    continue
                n0, n1, n2 = self.shape[t]
                o = self.off[t]
                if (a, b) == (0, 1):
                    task = _task(n0 * n1, n2, ("w", o), n2, segs)
                elif (a, b) == (1, 2):
                    task = _task(n0, n1 * n2, ("w", o), n1 * n2, segs)
                else:
                    task = _task(n1, n0 * n2, ("w102", o), n0 * n2, segs)
                task["role"] = "pair"
                self.launches[0].append(task)

    def _trimers(self, avail):
        """Three-stage products of every trimer charge block (build_H.py:103-188)."""
        ns, N = self.ns, self.Ns
        P_off, T1_off, T2_off, R3_off = {}, {}, {}, {}
        out_tasks = {}
        self.integral_keys = set()          # (kind, order) of every W matrix the stage-1 tasks read
        self.n_trimer_blocks = 0
        for ci in self.triples:
            for cj in self.triples:
                case = _case(ci, cj)
                if case is None:
                    continue
                kind, order, ops, _vfr = case
                x, y, z = order
                if not all(avail(order[k], ops[k], ci[order[k]], cj[order[k]]) for k in range(3)):
                    continue
                self.n_trimer_blocks += 1
                out_order = (x, z, y)
                self.orders_v.add(order)
                self.orders_w.add(out_order)
                nx, nxp = ns[x][ci[x]], ns[x][cj[x]]
                ny, nyp = ns[y][ci[y]], ns[y][cj[y]]
                nz, nzp = ns[z][ci[z]], ns[z][cj[z]]
                Ny, Nz = N[y], N[z]
                Kx = N[x] * N[x]
                # stage 1 (per build): Pt[x'][x][r][s] = a_k sum_k R1[x,x',k] W[(r,s),k] (+ delta U/4),
                # a_k = 4 (tex) or 2: the magnitude of the block factor (its sign goes to stage B)
                pkey = (kind, order, ci[x], cj[x])
                amag = 4.0 if kind == "tex" else 2.0
                if pkey not in P_off:
                    self.integral_keys.add((kind, order))
                    P_off[pkey] = self._alloc("Pt", nxp * nx * Ny * Nz)
                    segs = [_seg((("rho", x, ops[0], ci[x], cj[x]), 0), Kx, (("W", kind, order), 0), Kx, Kx,
                                 alpha=amag, sA=nxp * Kx)]
                    if kind == "tex":
                        segs.append(_seg((("eye", nx), 0), 1, (("Uq", order), 0), 1, 1, alpha=amag, sA=nx))
                    self.build_tasks.append(_task(nxp, Ny * Nz, ("Pt", P_off[pkey]), nx * Ny * Nz, segs, mode=0,
                                                  batch=nx, sC=Ny * Nz))
                # R3 as [z][s][z'] (per build)
                rkey = (z, ops[2], ci[z], cj[z])
                if rkey not in R3_off:
                    R3_off[rkey] = self._alloc("R3t", nz * Nz * nzp)
                    self.permutes.append(((("rho",) + rkey, 0), (nz, nzp, Nz), (0, 2, 1), ("R3t", R3_off[rkey])))
                # A: T1[(x' y')][(z s)] = sum_z' v_xyz[(x' y')][z'] R3t[(z s)][z']
                t1key = (order, cj, rkey)
                if t1key not in T1_off:
                    T1_off[t1key] = self._alloc("T1", nxp * nyp * nz * Nz)
                    task = _task(nxp * nyp, nz * Nz, ("T1", T1_off[t1key]), nz * Nz,
                                 [_seg((_vname(order), self.off[cj]), nzp, ("R3t", R3_off[rkey]), nzp, nzp)], mode=0)
                    task["role"] = "A"
                    self.launches[0].append(task)
                # B: T2p[x][z][y'][r] = sgn sum_x' sum_s T1[x'][y'][z][s] Pt[x'][x][r][s], written by the
                # GEMM's scatter epilogue (mode 2) straight into the K-contiguous layout of stage C:
                # output (m = (y', z), n = (x, r)) goes to (z nyp Ny + y' Ny) + (x nz nyp Ny + r), so
                # the lanes of a warp (consecutive n) store consecutive r
                s2 = -1.0 if (self.n_elec[1] - ci[1]) % 2 else 1.0
                s3 = -1.0 if (self.n_elec[2] - ci[2]) % 2 else 1.0
                sgn = _phase(kind, order, s2, s3)
                t2key = (pkey, t1key)            # one charge block: (ci[x], ci[z], cj) fix ci[y]
                if t2key not in T2_off:
                    T2_off[t2key] = self._alloc("T2p", nx * Ny * nyp * nz)
                    p0, q0 = P_off[pkey], T1_off[t1key]
                    segs = [_seg(("T1", q0 + xp * nyp * nz * Nz), Nz, ("Pt", p0 + xp * nx * Ny * Nz), Nz, Nz,
                                 alpha=sgn)
                            for xp in range(nxp)]
                    task = _task(nyp * nz, nx * Ny, ("T2p", T2_off[t2key]), 1, segs, mode=2)
                    yi, zi = np.divmod(np.arange(nyp * nz), nz)
                    xi, ri = np.divmod(np.arange(nx * Ny), Ny)
                    task["maps"] = (zi * (nyp * Ny) + yi * Ny, np.zeros(nyp * nz, dtype=np.int64),
                                    xi * (nz * nyp * Ny) + ri, np.zeros(nx * Ny, dtype=np.int64))
                    task["role"] = "B"
                    self.launches[1].append(task)
                # C: w_xzy[(x z)][y] += sum_(y',r) T2p[(x z)][(y' r)] R2[y][(y' r)]
                okey = (out_order, ci)
                if okey not in out_tasks:
                    out_tasks[okey] = _task(nx * nz, ny, (_wname(out_order), self.off[ci]), ny, [])
                    out_tasks[okey]["role"] = "C"
                    self.launches[2].append(out_tasks[okey])
                out_tasks[okey]["segs"].append(_seg(("T2p", T2_off[t2key]), nyp * Ny,
                                                    (("rho", y, ops[1], ci[y], cj[y]), 0), nyp * Ny, nyp * Ny))

    # ---------------------------------------------------------------------------------
    def permutation(self, order):
        """Gather index of the copy of v in fragment order `order`: v_order = v[idx]; the
        permuted accumulator goes back with w[idx] += w_order."""
        idx = np.empty(self.dim, dtype=np.int64)
        for t in self.triples:
            o, sh = self.off[t], self.shape[t]
            n = int(np.prod(sh))
            idx[o:o + n] = o + np.arange(n).reshape(sh).transpose(order).ravel()
        return idx

    def product_index(self):
        """Position of every vector element in the reference's product order
        (I0 I1 I2 row-major over the three fragments' charge-blocked state lists)."""
        offs, tots = [], []
        for f in range(3):
            acc, o = 0, {}
            for c in self.charges[f]:
                o[c] = acc
                acc += self.ns[f][c]
            offs.append(o)
            tots.append(acc)
        idx = np.empty(self.dim, dtype=np.int64)
        for t in self.triples:
            n0, n1, n2 = self.shape[t]
            i0, i1, i2 = np.meshgrid(np.arange(n0), np.arange(n1), np.arange(n2), indexing="ij")
            g = ((offs[0][t[0]] + i0) * tots[1] + offs[1][t[1]] + i1) * tots[2] + offs[2][t[2]] + i2
            idx[self.off[t]:self.off[t] + n0 * n1 * n2] = g.ravel()
        return idx, tots[0] * tots[1] * tots[2]


def _task_flops(t):
    return sum(2.0 * t["M"] * t["N"] * s["K"] * t["batch"] for s in t["segs"])


def trimer_integral_matrices(V, U, order_kinds, Ns):
    """W[(kind, order)] = the V block of the case with R1's indices last, (Ny Nz, Nx Nx)
    (as trimer.XRTrimerPlan), and Uq[order] = U[x,y,z] / 4 for the Ex1min1pls cases;
    V(m,n,o,p) and U(k,m,n) return torch tensors or NumPy arrays."""
    W, Uq = {}, {}
    for kind, order in sorted(order_kinds):
        x, y, z = order
        Nx, Ny, Nz = Ns[x], Ns[y], Ns[z]
        if kind == "t2m":        # V[x,x,y,z] = V[p,q,r,s], R1 indexed (q, p)
            Vb, ax = V(x, x, y, z), (2, 3, 1, 0)
        elif kind == "t2p":      # V[y,z,x,x] = V[r,s,p,q], R1 indexed (q, p)
            Vb, ax = V(y, z, x, x), (0, 1, 3, 2)
        else:                    # V[x,y,x,z] = V[p,r,q,s], R1 indexed (p, q)
            Vb, ax = V(x, y, x, z), (1, 3, 0, 2)
        Wt = Vb.permute(*ax) if hasattr(Vb, "permute") else Vb.transpose(ax)
        W[(kind, order)] = Wt.reshape(Ny * Nz, Nx * Nx)
        if kind == "tex":
            Uq[order] = 0.25 * U(x, y, z).reshape(Ny * Nz, 1)
    return W, Uq


def permute_tasks(ops):
    """xrh_permute_task records (host) for ops = [(src address, shape, ax, dst address,
    scale)]: dst = scale * src.reshape(shape).transpose(ax), row-major.  Returns (table,
    total elements)."""
    tab = np.zeros(len(ops), dtype=_lib.PERMUTE_TASK_DTYPE)
    begin = 0
    for i, (src, shape, ax, dst, scale) in enumerate(ops):
        if len(shape) > 6:
            raise ValueError("permutes of more than 6 indices")
        n = int(np.prod(shape))
        strides = np.ones(len(shape), dtype=np.int64)
        for k in range(len(shape) - 2, -1, -1):
            strides[k] = strides[k + 1] * shape[k + 1]
        e = tab[i]
        e["src"], e["dst"], e["ndim"], e["scale"] = src, dst, len(shape), float(scale)
        for k, a in enumerate(ax):
            e["dst_shape"][k] = shape[a]
            e["src_stride"][k] = strides[a]
        e["elem_begin"], e["n_elems"] = begin, n
        begin += n
    return tab, begin


class _PairIntegrals:
    """The integral accessors of fragments (a, b) of a larger system, numbered (0, 1)."""

    def __init__(self, ints, frags):
        self.ints, self.f = ints, tuple(frags)

    def T(self, m, n):
        return self.ints.T(self.f[m], self.f[n])

    def U(self, k, m, n):
        return self.ints.U(self.f[k], self.f[m], self.f[n])

    def V(self, m, n, o, p):
        return self.ints.V(self.f[m], self.f[n], self.f[o], self.f[p])


class XRTrimerHamiltonian:
    """w = H v for the order-0 general-XRCC Hamiltonian of three fragments on the device.

    spaces:       three FragmentSpace objects;  n_states: three {charge: n};  charges: three lists
    ints:         DeviceIntegrals over the three fragments (T, U, V block accessors)
    precision:    arithmetic of the pair builds (XRDimerPlan: 'fp64', 'bf16x3', 'tf32x3')
    hv_precision: arithmetic of the H x v GEMMs: 'fp64'; 'fp32' (FP32 products, FP64 sums); or
                  'tf32x3' / 'bf16x3' (the dominant stage on the tensor cores in split precision,
                  the rest with FP32 products and FP64 sums)
    total_charge: restrict the vector to one total charge (None: the whole product space)
    pair_output:  'split' (pair plans hold the dimer couplings H2) or 'full' (they hold the
                  full pair Hamiltonians, which then also serve pair energies and their reverse
                  pass; the monomer terms of the product enter with factor -1)
    builders:     three DensityBuilder objects to use instead of the object's own
    pair_terms_tc: split forms only: the pair terms of the product on the tensor cores (True;
                  the pair sector matrices are then held a second time as split copies) or
                  with FP32 products and FP64 sums on the CUDA cores (False, no copies)

    build(coeffs) runs the three pair builds (densities, monomer and dimer blocks) and the
    per-build trimer stage; apply(x) then returns H x as a device vector in block layout
    (product_index() maps it to the reference's product order).  Nothing is
    allocated after construction: every launch reads persistent buffers through task tables
    uploaded once, so a build or a product can be captured in a CUDA graph."""

    def __init__(self, spaces, n_states, charges, ints, precision="fp64", hv_precision="fp64", total_charge=None,
                 autotune=True, pair_output="split", builders=None, pair_terms_tc=True):
        from .densities import DensityBuilder
        from .hamiltonian import XRDimerPlan
        if pair_output not in ("split", "full"):
            raise ValueError("pair_output must be 'split' or 'full'")
        dev = spaces[0].device
        self.device = dev
        self.charges = [list(c) for c in charges]
        self.n_states = [dict(n) for n in n_states]
        self.pair_output = pair_output
        # one density builder per fragment, shared by the two pair plans that hold it (FP32
        # products on the split-precision paths, as XRDimerPlan chooses for its own)
        dens_precision = "fp32" if precision in ("bf16x3", "tf32x3") else "fp64"
        self.builders = list(builders) if builders is not None else [
            DensityBuilder(spaces[f], self.n_states[f], precision=dens_precision) for f in range(3)]
        # pair sectors a restricted vector reaches: total charge minus the spectator's charge
        pair_sectors = [None] * 3
        if total_charge is not None:
            for p, (a, b) in enumerate(PAIRS):
                s_ = 3 - a - b
                pair_sectors[p] = sorted({total_charge - c for c in self.charges[s_]})
        # the three pair plans share one split registry: each fragment's densities are split once
        from .gemm import SplitRegistry
        self.pair_registry = SplitRegistry(precision, dev) if precision in ("bf16x3", "tf32x3") else None
        self.plans = [XRDimerPlan([spaces[a], spaces[b]], [self.n_states[a], self.n_states[b]],
                                  [self.charges[a], self.charges[b]], _PairIntegrals(ints, (a, b)), output=pair_output,
                                  precision=precision, convention="general", layout="sector", autotune=autotune,
                                  builders=[self.builders[a], self.builders[b]], total_charges=pair_sectors[p],
                                  registry=self.pair_registry)
                      for p, (a, b) in enumerate(PAIRS)]
        # each fragment's coefficient buffers and monomer blocks from one pair plan that holds it
        holder = {0: (0, 0), 1: (0, 1), 2: (1, 1)}
        self.rho = [b.rho for b in self.builders]
        self.coeffs = [self.plans[p].coeffs[k] for p, k in (holder[f] for f in range(3))]
        self.H1blk = [self.plans[p].H1blk[k] for p, k in (holder[f] for f in range(3))]

        def avail(f, op, bc, kc):
            return (bc, kc) in self.rho[f].get(op, {})

        plan = TrimerHvPlan(self.charges, self.n_states, [sp.n_elec_ref for sp in spaces], [sp.N for sp in spaces],
                            avail, total_charge, monomer_scale=-1.0 if pair_output == "full" else 1.0)
        if plan.dim == 0:
            raise ValueError(f"no product state has total charge {total_charge}")
        self.plan = plan
        self.total_charge = total_charge
        for p, lay in enumerate(plan.pair_layout):
            for t, (base, dimt) in lay.items():
                if t not in self.plans[p].sectors:
                    continue            # a sector the restricted vector never reaches
                sec = self.plans[p].sectors[t]
                assert sec["dim"] == dimt and sec["base"] == base, "pair sector layout mismatch"
        f64 = dict(dtype=torch.float64, device=dev)
        self.bufs = {k: torch.zeros(max(int(n), 1), **f64) for k, n in plan.sizes.items()}
        W, Uq = trimer_integral_matrices(ints.V, ints.U, plan.integral_keys, plan.Ns)
        self.W = {k: w.contiguous().reshape(-1) for k, w in W.items()}
        self.Uq = {k: u.contiguous().reshape(-1) for k, u in Uq.items()}
        self.eyes = {}
        self._gather = {o: torch.as_tensor(plan.permutation(o), device=dev) for o in sorted(plan.orders_v - {IDENTITY})}
        # w += w_order[inverse permutation]: every permuted accumulator returns in one gather-sum
        self._scatter = {}
        for o in sorted(plan.orders_w - {IDENTITY}):
            idx = plan.permutation(o)
            inv = np.empty_like(idx)
            inv[idx] = np.arange(len(idx))
            self._scatter[o] = torch.as_tensor(inv, device=dev)
        if len(self._scatter) > 8:
            raise ValueError("more than 8 permuted accumulators")
        terms = np.zeros(1, dtype=_lib.GATHER_TERMS_DTYPE)
        for t, (o, inv) in enumerate(self._scatter.items()):
            terms[0]["src"][t] = self.bufs[_wname(o)].data_ptr()
            terms[0]["idx"][t] = inv.data_ptr()
        terms[0]["n_terms"] = len(self._scatter)
        self._scatter_terms = terms
        self._permutes = self._permute_table([(self._resolve(src), shape, ax, self._resolve(dst), 1.0)
                                              for src, shape, ax, dst in plan.permutes])
        self._mid_permutes = self._permute_table([(self._resolve(src), shape, ax, self._resolve(dst), a)
                                                  for src, shape, ax, dst, a in plan.mid_permutes])
        # split forms: the pair terms and the three trimer stages on the tensor cores, each role
        # with its own split registry (a vector block is an operand of several shapes); operands
        # that change per product (vector blocks, T1, T2p) are split per product, the rest once
        # per build; the monomer terms and the per-build stage keep FP32 products / FP64 sums
        self.tc = hv_precision in ("bf16x3", "tf32x3")
        simt = "fp32" if self.tc else hv_precision
        tc_roles = (("pair",) if pair_terms_tc else ()) + ("A", "B", "C") if self.tc else ()
        self.stage1 = self._grouped(plan.build_tasks, simt)
        self.simt = [self._grouped([t for t in L if t.get("role") not in tc_roles], simt) for L in plan.launches]
        self.tcs = [[] for _ in plan.launches]
        self.stage_b = self.simt[1]
        if self.tc:
            from .gemm import SplitRegistry, TCGroupedGemm
            per_product = ("v", "T1", "T2p")
            for k, L in enumerate(plan.launches):
                for role in tc_roles:
                    tasks = [t for t in L if t.get("role") == role]
                    if not tasks:
                        continue
                    reg = SplitRegistry(hv_precision, dev)
                    g = TCGroupedGemm(reg)
                    for t in tasks:
                        assert t["batch"] == 1 and all(sg["flags"] == 0 for sg in t["segs"])
                        segs, groups = [], []
                        for sg in t["segs"]:
                            segs.append((self._resolve(sg["A"]), sg["lda"], self._resolve(sg["B"]), sg["ldb"], sg["K"],
                                         sg["alpha"]))
                            groups.append(tuple("product" if isinstance(r[0], str) and r[0].startswith(per_product)
                                                else "build" for r in (sg["A"], sg["B"])))
                        g.add(t["M"], t["N"], segs, self._resolve(t["C"]), t["ldc"], mode=t["mode"], groups=groups,
                              maps=self._maps(t))
                    reg.upload()
                    g.finalize()
                    if autotune:
                        g.autotune()
                    self.tcs[k].append((reg, g))
                    if role == "B":
                        self.stage_b = g
        self.flops_apply = plan.flops_apply
        self.dim = plan.dim

    # ---------------------------------------------------------------------------------
    def _ext(self, key):
        kind = key[0]
        if kind == "rho":
            _, f, op, bc, kc = key
            return self.rho[f][op][(bc, kc)].reshape(-1)
        if kind == "H1":
            return self.H1blk[key[1]][key[2]].reshape(-1)
        if kind == "H2":
            return self.plans[key[1]].sectors[key[2]]["H"].reshape(-1)
        if kind == "W":
            return self.W[(key[1], key[2])]
        if kind == "Uq":
            return self.Uq[key[1]]
        if kind == "eye":
            n = key[1]
            if n not in self.eyes:
                self.eyes[n] = torch.eye(n, dtype=torch.float64, device=self.device).reshape(-1)
            return self.eyes[n]
        return self.bufs[key]

    def _resolve(self, ref):
        buf, off = ref
        t = self._ext(buf)
        return t[off:]

    def _maps(self, t):
        """Device index maps of a mode-2 (scatter) record: (rowA, colA, rowB, colB) as int32 and
        zero diagonal flags (no delta terms)."""
        if t["mode"] != 2:
            return None
        dev = self.device
        rowA, colA, rowB, colB = (torch.as_tensor(np.asarray(a, dtype=np.int32), device=dev) for a in t["maps"])
        return (rowA, colA, rowB, colB, torch.zeros(t["M"], dtype=torch.uint8, device=dev),
                torch.zeros(t["N"], dtype=torch.uint8, device=dev))

    def _grouped(self, tasks, precision):
        g = GroupedGemm(self.device, precision=precision)
        for t in tasks:
            segs = []
            for s in t["segs"]:
                segs.append((self._resolve(s["A"]), s["lda"], self._resolve(s["B"]), s["ldb"], s["K"], s["alpha"],
                             s["flags"], s["sA"], s["sB"]))
            g.add(t["M"], t["N"], segs, self._resolve(t["C"]), t["ldc"], mode=t["mode"], batch=t["batch"], sC=t["sC"],
                  maps=self._maps(t))
        return g.finalize()

    # ---------------------------------------------------------------------------------
    def trimer_integral_set(self, ints):
        """Device copies of the per-build trimer integral matrices (W, Uq) for these three
        fragments' integrals, for load_integral_sets."""
        W, Uq = trimer_integral_matrices(ints.V, ints.U, self.plan.integral_keys, self.plan.Ns)
        return {"W": {k: w.contiguous().reshape(-1) for k, w in W.items()},
                "Uq": {k: u.contiguous().reshape(-1) for k, u in Uq.items()}}

    def load_integral_sets(self, pair_sets, trimer_set):
        """New integrals from prepared sets (XRDimerPlan.integral_set of each pair, in PAIRS
        order, and trimer_integral_set): device copies and operand splits only."""
        for pl, S in zip(self.plans, pair_sets):
            pl.load_integral_set(S)
        for k, w in self.W.items():
            w.copy_(trimer_set["W"][k])
        for k, u in self.Uq.items():
            u.copy_(trimer_set["Uq"][k])

    def set_coeffs(self, coeffs):
        """coeffs: three {charge: CUDA float64 (n_states, n_conf)} dicts."""
        for p, (a, b) in enumerate(PAIRS):
            self.plans[p].set_coeffs([coeffs[a], coeffs[b]])

    def build(self, coeffs=None):
        """Enqueue the pair builds and the per-build trimer stage (no host synchronisation)."""
        if coeffs is not None:
            self.set_coeffs(coeffs)
        for b, z in zip(self.builders, self.coeffs):
            b.build(z)
        if self.pair_registry is not None:
            for b in self.builders:
                self.pair_registry.split(b.split_group)
        for pl in self.plans:
            pl.launch(build_densities=False, split_inputs=False)
        self._run_permutes(self._permutes)
        self.stage1.run()
        for phase in self.tcs:
            for reg, _g in phase:
                reg.split("build")

    def _permute_table(self, ops):
        """xrh_permute_grouped task table: dst = scale * src.view(shape).permute(ax)."""
        tab, total = permute_tasks([(src.data_ptr(), shape, ax, dst.data_ptr(), scale)
                                    for src, shape, ax, dst, scale in ops])
        dev_tab = torch.from_numpy(tab.view(np.uint8).copy()).to(self.device) if len(ops) else None
        return (dev_tab, len(ops), total)

    @staticmethod
    def _run_permutes(table):
        tab, n_t, total = table
        if n_t:
            call("xrh_permute_grouped", ptr(tab), n_t, total, stream_ptr())

    def apply(self, x, out=None):
        """out = H x (device vectors of length self.dim, block layout); returns out."""
        v, w = self.bufs["v"], self.bufs["w"]
        s = stream_ptr()
        if x.data_ptr() != v.data_ptr():
            v.copy_(x)
        _lib.zero_(w)
        for o in self._scatter:
            _lib.zero_(self.bufs[_wname(o)])
        for o, idx in self._gather.items():
            call("xrh_index_move", idx.numel(), ptr(idx), ptr(v), ptr(self.bufs[_vname(o)]), 1, s)
        for k in range(3):
            if k == 2:
                self._run_permutes(self._mid_permutes)
            self.simt[k].run()
            for reg, g in self.tcs[k]:
                reg.split("product")
                g.run()
        if self._scatter:
            call("xrh_gather_sum", self.dim, self._scatter_terms.ctypes.data, ptr(w), 1, s)
        if out is not None and out.data_ptr() != w.data_ptr():
            out.copy_(w)
            return out
        return w

    def check_status(self):
        """Raise if a bounded device wait of a tensor-core launch timed out (syncs)."""
        for pl in self.plans:
            pl.check_status()
        for phase in self.tcs:
            for _reg, g in phase:
                g.check()

    def product_index(self):
        """(device int64 index, product-space dimension): element e of a block-layout vector is
        element idx[e] of the vector in the reference's product order."""
        idx, dim = self.plan.product_index()
        return torch.as_tensor(idx, device=self.device), dim

    def lowest(self, k=1, m=60, seed=7, tol=None, max_restarts=30, graph=False, v0=None):
        """Lowest k eigenvalues (FP64 Lanczos on the matrix-free product) and the residual
        estimate of the lowest; the ground-state vector is self.lanczos.ground_vector().
        tol: restart the Krylov loop from the current ground Ritz vector until the residual
        of the lowest pair is below tol * max(1, |E0|) (None: one loop of m steps).
        graph: replay the m-step Krylov loop (products and Gram-Schmidt) as one CUDA graph,
        captured on the first call.
        v0: start vector (device, length self.dim); default: the seeded random start on the
        first call, the last ground vector on later calls."""
        from .eigen import Lanczos
        if getattr(self, "lanczos", None) is None or self.lanczos.m != min(m, self.dim):
            self.lanczos = Lanczos(self.dim, m=m, device=self.device, seed=seed, mode="steps")
            self._krylov_graph = None
        lz = self.lanczos

        def krylov():
            lz.krylov_operator(lambda x, y: self.apply(x, y))

        if graph and self._krylov_graph is None:
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            v0 = lz.v0.clone()
            with torch.cuda.stream(s):          # warm the allocator outside the capture
                krylov()
            torch.cuda.current_stream().wait_stream(s)
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                krylov()
            lz.v0.copy_(v0)
            self._krylov_graph = g
        if v0 is not None:
            lz.v0.copy_(v0)
        w = resid = None
        self.lanczos_cycles = 0
        for _ in range(max_restarts if tol is not None else 1):
            self.lanczos_cycles += 1
            if graph:
                self._krylov_graph.replay()
            else:
                krylov()
            lz.stage_to_host()
            torch.cuda.current_stream().synchronize()
            w, resid = lz.solve(k)
            if tol is None or resid <= tol * max(1.0, abs(float(w[0]))):
                break
            lz.v0.copy_(lz.ground_vector())
        return w, resid
