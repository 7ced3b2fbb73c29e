"""numpy restatement of ugacc's RHF-CC hot path (test infrastructure; see package doc).

Index conventions follow the reference: occupied i,j,k,l,m,n,o; virtual a,b,c,d,e,f,g.
``V('ovvv')[m,a,e,f]`` is the reference's ``ints[m][a+no][e+no][f+no] = <ma|ef>`` and
``L(...)`` is its ``L = 2<pq|rs> - <pq|sr>`` (hamiltonian.cc:88, :96-102).  Blocks are
formed from the density-fitting factors, so no [nact]^4 array is ever built.
"""
from __future__ import annotations

import math
from functools import partial

import numpy as np

ein = partial(np.einsum, optimize=True)


# --------------------------------------------------------------------------------------
# Hamiltonian blocks                                          (hamiltonian.cc:43-102)
# --------------------------------------------------------------------------------------
class Hamiltonian:
    def __init__(self, ham):
        self.no, self.nv = ham.no, ham.nv
        self.nact = ham.no + ham.nv
        self.f = np.diag(ham.eps).astype(np.float64)
        self.B = ham.B
        self._cache = {}

    def _rng(self, c):
        return slice(0, self.no) if c == "o" else slice(self.no, self.nact)

    def V(self, s: str) -> np.ndarray:
        """<pq|rs> block, e.g. V('oovv')[i,j,a,b] = <ij|ab> = (ia|jb)."""
        if s not in self._cache:
            p, q, r, t = (self._rng(c) for c in s)
            self._cache[s] = np.ascontiguousarray(ein("Qpr,Qqs->pqrs", self.B[:, p, r], self.B[:, q, t]))
        return self._cache[s]

    def L(self, s: str) -> np.ndarray:
        """L[p,q,r,s] = 2<pq|rs> - <pq|sr> restricted to the block s."""
        key = "L" + s
        if key not in self._cache:
            swapped = self.V(s[0] + s[1] + s[3] + s[2]).transpose(0, 1, 3, 2)
            self._cache[key] = np.ascontiguousarray(2.0 * self.V(s) - swapped)
        return self._cache[key]

    def fblk(self, s: str) -> np.ndarray:
        return self.f[self._rng(s[0]), self._rng(s[1])]


# --------------------------------------------------------------------------------------
# DIIS: circular 8-slot Pulay extrapolation, B scaled by max|B|, -1 border
# (the procedure of attic/diis.cc:13-161, used at ccwfn.cc:217-221)
# --------------------------------------------------------------------------------------
class DIIS:
    def __init__(self, nmax: int = 8):
        self.nmax = nmax
        self.err: list[np.ndarray] = []
        self.vec: list[np.ndarray] = []
        self.nadded = 0

    def add(self, err: np.ndarray, vec: np.ndarray) -> None:
        if len(self.err) < self.nmax:
            self.err.append(err.copy())
            self.vec.append(vec.copy())
        else:
            slot = self.nadded % self.nmax
            self.err[slot] = err.copy()
            self.vec[slot] = vec.copy()
        self.nadded += 1

    def size(self) -> int:
        return len(self.err)

    def extrapolate(self) -> np.ndarray:
        n = len(self.err)
        E = np.array(self.err)
        B = np.zeros((n + 1, n + 1))
        B[:n, :n] = E @ E.T
        mx = np.abs(B[:n, :n]).max()
        if mx > 0:
            B[:n, :n] /= mx
        B[:n, n] = B[n, :n] = -1.0
        rhs = np.zeros(n + 1)
        rhs[n] = -1.0
        c = np.linalg.solve(B, rhs)
        return np.tensordot(c[:n], np.array(self.vec), axes=1)


def _pack(x1, x2):
    return np.concatenate([x1.ravel(), x2.ravel()])


def _unpack(v, like1, like2):
    n1 = like1.size
    return v[:n1].reshape(like1.shape).copy(), v[n1:].reshape(like2.shape).copy()


class NotConverged(RuntimeError):
    """Raised like the reference's PSIEXCEPTION("Computation has not converged.")."""


# --------------------------------------------------------------------------------------
# Ground state                                                              (ccwfn.cc)
# --------------------------------------------------------------------------------------
class CCWfn:
    def __init__(self, H: Hamiltonian, maxiter: int = 100, r_convergence: float = 1e-7, diis: bool = True):
        self.H = H
        self.maxiter, self.conv, self.do_diis = maxiter, r_convergence, diis
        no, nv = H.no, H.nv
        eo = np.diag(H.f)[:no]
        ev = np.diag(H.f)[no:]
        # denominators and MP2 guess, ccwfn.cc:62-87
        self.D1 = eo[:, None] - ev[None, :]
        self.D2 = eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None] - ev[None, None, None, :]
        self.t1 = H.fblk("ov") / self.D1
        self.t2 = H.V("oovv") / self.D2
        self.build_tau()
        self.iter_energies: list[float] = []
        self.iterations = 0

    def build_tau(self):  # ccwfn.cc:284-298
        t1t1 = ein("ia,jb->ijab", self.t1, self.t1)
        self.tau = self.t2 + t1t1
        self.ttau = self.t2 + 0.5 * t1t1

    def energy(self):  # ccwfn.cc:260-282
        H = self.H
        # the one-electron loop assigns instead of accumulating (ccwfn.cc:272): only the
        # last (i,a) pair survives
        one = 2.0 * H.fblk("ov")[-1, -1] * self.t1[-1, -1]
        two = ein("ijab,ijab->", self.tau, H.L("oovv"))
        return one + two

    def build_F(self, t1, ttau):  # ccwfn.cc:311-356
        H = self.H
        fov = H.fblk("ov")
        Fvv = H.fblk("vv").copy()
        Fvv -= 0.5 * ein("me,ma->ae", fov, t1)
        Fvv += ein("mf,mafe->ae", t1, H.L("ovvv"))
        Fvv -= ein("mnaf,mnef->ae", ttau, H.L("oovv"))
        Foo = H.fblk("oo").copy()
        Foo += 0.5 * ein("ie,me->mi", t1, fov)
        Foo += ein("ne,mnie->mi", t1, H.L("ooov"))
        Foo += ein("inef,mnef->mi", ttau, H.L("oovv"))
        Fov = fov.copy()
        Fov += ein("nf,mnef->me", t1, H.L("oovv"))
        return Fvv, Foo, Fov

    def build_W(self, t1, t2, tau):  # ccwfn.cc:358-430
        H = self.H
        Woooo = H.V("oooo").copy()
        Woooo += ein("je,mnie->mnij", t1, H.V("ooov"))
        Woooo += ein("ie,mnej->mnij", t1, H.V("oovo"))
        Woooo += ein("ijef,mnef->mnij", tau, H.V("oovv"))
        X = 0.5 * t2 + ein("jf,nb->jnfb", t1, t1)
        Wovov = -H.V("ovov")
        Wovov -= ein("jf,mbfe->mbje", t1, H.V("ovvv"))
        Wovov += ein("nb,mnje->mbje", t1, H.V("ooov"))
        Wovov += ein("mnfe,jnfb->mbje", H.V("oovv"), X)
        Wovvo = H.V("ovvo").copy()
        Wovvo += ein("jf,mbef->mbej", t1, H.V("ovvv"))
        Wovvo -= ein("nb,mnej->mbej", t1, H.V("oovo"))
        Wovvo -= ein("mnef,jnfb->mbej", H.V("oovv"), X)
        Wovvo += 0.5 * ein("mnef,njfb->mbej", H.L("oovv"), t2)
        Zmbij = ein("mbef,ijef->mbij", H.V("ovvv"), tau)
        return Woooo, Wovov, Wovvo, Zmbij

    def build_t1(self, t1, t2, Fvv, Foo, Fov):  # ccwfn.cc:432-469
        H = self.H
        R = H.fblk("vo").T.copy()
        R += ein("ie,ae->ia", t1, Fvv)
        R -= ein("ma,mi->ia", t1, Foo)
        R += ein("imae,me->ia", 2.0 * t2 - t2.swapaxes(2, 3), Fov)
        R += ein("nf,nafi->ia", t1, H.L("ovvo"))
        R += ein("mief,maef->ia", 2.0 * t2 - t2.swapaxes(2, 3), H.V("ovvv"))
        R -= ein("mnae,nmei->ia", t2, H.L("oovo"))
        return R

    def build_t2(self, t1, t2, tau, Fvv, Foo, Fov, Woooo, Wovov, Wovvo, Zmbij):  # ccwfn.cc:471-539
        H = self.H
        R = H.V("oovv").copy()
        R += ein("ijae,be->ijab", t2, Fvv) + ein("jibe,ae->ijab", t2, Fvv)
        tF = ein("mb,me->be", t1, Fov)
        R -= 0.5 * (ein("ijae,be->ijab", t2, tF) + ein("ijeb,ae->ijab", t2, tF))
        R -= ein("imab,mj->ijab", t2, Foo) + ein("mjab,mi->ijab", t2, Foo)
        tF2 = ein("je,me->mj", t1, Fov)
        R -= 0.5 * (ein("imab,mj->ijab", t2, tF2) + ein("mjab,mi->ijab", t2, tF2))
        R += ein("mnab,mnij->ijab", tau, Woooo)
        R += ein("ijef,abef->ijab", tau, H.V("vvvv"))
        R += ein("ie,abej->ijab", t1, H.V("vvvo")) + ein("je,baei->ijab", t1, H.V("vvvo"))
        R -= ein("ma,mbij->ijab", t1, H.V("ovoo")) + ein("mb,maji->ijab", t1, H.V("ovoo"))
        t2a = t2 - t2.swapaxes(2, 3)
        R += ein("imae,mbej->ijab", t2a, Wovvo) + ein("jmbe,maei->ijab", t2a, Wovvo)
        R += ein("imae,mbej->ijab", t2, Wovvo + Wovov.transpose(0, 1, 3, 2))
        R += ein("jmbe,maei->ijab", t2, Wovvo + Wovov.transpose(0, 1, 3, 2))
        R += ein("mjae,mbie->ijab", t2, Wovov) + ein("imeb,maje->ijab", t2, Wovov)
        R -= ein("ie,ma,mbej->ijab", t1, t1, H.V("ovvo"))
        R -= ein("ie,mb,maje->ijab", t1, t1, H.V("ovov"))
        R -= ein("je,ma,mbie->ijab", t1, t1, H.V("ovov"))
        R -= ein("je,mb,maei->ijab", t1, t1, H.V("ovvo"))
        R -= ein("ma,mbij->ijab", t1, Zmbij) + ein("mb,maji->ijab", t1, Zmbij)
        return R

    def t1norm(self):  # ccwfn.cc:541-553
        return math.sqrt((self.t1 ** 2).sum() / (2 * self.H.no))

    def iterate_once(self):
        """One pass of the loop body ccwfn.cc:210-215 (without the DIIS step)."""
        t1, t2, tau, ttau = self.t1, self.t2, self.tau, self.ttau
        Fvv, Foo, Fov = self.build_F(t1, ttau)
        W = self.build_W(t1, t2, tau)
        R1 = self.build_t1(t1, t2, Fvv, Foo, Fov)
        R2 = self.build_t2(t1, t2, tau, Fvv, Foo, Fov, *W)
        rms = math.sqrt((R1 ** 2).sum() + (R2 ** 2).sum())  # ccwfn.cc:555-582
        return t1 + R1 / self.D1, t2 + R2 / self.D2, rms

    def compute_energy(self):  # ccwfn.cc:188-258 (CCSD part)
        self.emp2 = self.energy()
        diis = DIIS(8)
        eccsd = float("nan")
        rms = float("inf")
        for it in range(1, self.maxiter + 1):
            told1, told2 = self.t1, self.t2
            self.t1, self.t2, rms = self.iterate_once()
            self.iterations = it
            if rms < self.conv:
                break
            if self.do_diis:
                diis.add(_pack(self.t1 - told1, self.t2 - told2), _pack(self.t1, self.t2))
                if diis.size() > 2:
                    self.t1, self.t2 = _unpack(diis.extrapolate(), self.t1, self.t2)
            self.build_tau()
            eccsd = self.energy()
            self.iter_energies.append(eccsd)
        self.build_tau()
        self.build_tstar()
        if rms >= self.conv:
            raise NotConverged("Computation has not converged.")
        self.eccsd = eccsd
        return eccsd

    def build_tstar(self):  # ccwfn.cc:628-645
        self.t1s = 2.0 * self.t1
        self.t2s = 4.0 * self.t2 - 2.0 * self.t2.swapaxes(2, 3)

    # ---------------------------------------------------------------- (T)
    def W3_ijk(self, i, j, k):  # ccwfn.cc:1388-1418
        H, t2 = self.H, self.t2
        Vovvv, Vooov = H.V("ovvv"), H.V("ooov")

        def ct(X, Y, perm):
            """sum_e X[x,e] Y[e,u,v] as one matrix product, indexed [x,u,v] and then
            transposed to [a,b,c] by perm"""
            n0, n1, n2 = X.shape[0], Y.shape[1], Y.shape[2]
            return (X @ Y.reshape(Y.shape[0], n1 * n2)).reshape(n0, n1, n2).transpose(perm)

        # each e-sum shares its output ordering with one m-sum: one transposed add per pair
        pairs = [((t2[k, j], Vovvv[i]), (Vooov[j, k].T, t2[i]), (1, 2, 0)),  # eab,ce / mc,mab -> abc
                 ((t2[j, k], Vovvv[i]), (Vooov[k, j].T, t2[i]), (1, 0, 2)),  # eac,be / mb,mac
                 ((t2[j, i], Vovvv[k]), (Vooov[i, j].T, t2[k]), (2, 0, 1)),  # eca,be / mb,mca
                 ((t2[i, j], Vovvv[k]), (Vooov[j, i].T, t2[k]), (0, 2, 1)),  # ecb,ae / ma,mcb
                 ((t2[i, k], Vovvv[j]), (Vooov[k, i].T, t2[j]), (0, 1, 2)),  # ebc,ae / ma,mbc
                 ((t2[k, i], Vovvv[j]), (Vooov[i, k].T, t2[j]), (2, 1, 0))]  # eba,ce / mc,mba
        W = None
        for (Xe, Ye), (Xm, Ym), perm in pairs:
            G = ct(Xe, Ye, (0, 1, 2))
            G -= ct(Xm, Ym, (0, 1, 2))
            if W is None:
                W = np.ascontiguousarray(G.transpose(perm))
            else:
                W += G.transpose(perm)
        return W

    # the six orderings of (a,b,c) that the energy expression reads, as the positions of
    # the triple that index W3: (0,2,1) is W3[a][c][b], (2,0,1) is W3[c][a][b], and so on
    PERMS = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (2, 0, 1), (1, 2, 0), (2, 1, 0)]

    def tuple_setup(self):
        """What every (T) tuple term uses, on the a >= b >= c triples only (in C order):
        the occupied energies, the triples (a,b,c), the degeneracy divisor
        1 + [a==b] + [a==c] + [b==c] and e_a + e_b + e_c."""
        H = self.H
        no, nv = H.no, H.nv
        eo = np.diag(H.f)[:no]
        ev = np.diag(H.f)[no:]
        a_, b_, c_ = np.meshgrid(np.arange(nv), np.arange(nv), np.arange(nv), indexing="ij")
        a, b, c = np.nonzero((a_ >= b_) & (b_ >= c_))
        deg = 1.0 + (a == b) + (a == c) + (b == c)
        dv = ev[a] + ev[b] + ev[c]
        return eo, (a, b, c), deg, dv

    def tcorr_tuple(self, i, j, k, setup=None):  # ccwfn.cc:813-849: the term of one i >= j >= k
        H, t1 = self.H, self.t1
        nv = H.nv
        Voovv = H.V("oovv")
        eo, abc, deg, dv = setup if setup is not None else self.tuple_setup()
        Wf = self.W3_ijk(i, j, k).ravel()
        Vij, Vik, Vjk = Voovv[i, j], Voovv[i, k], Voovv[j, k]
        P, Q = {}, {}
        for p in self.PERMS:  # W3 and V3 at (x,y,z) = the triple in ordering p
            x, y, z = abc[p[0]], abc[p[1]], abc[p[2]]
            w = Wf[(x * nv + y) * nv + z]
            P[p] = w
            Q[p] = (w + Vij[x, y] * t1[k, z] + Vik[x, z] * t1[j, y] + Vjk[y, z] * t1[i, x]) / deg
        X3 = sum(P[p] * Q[p] for p in self.PERMS)
        Y3 = Q[(0, 1, 2)] + Q[(2, 0, 1)] + Q[(1, 2, 0)]  # V3[abc] + V3[cab] + V3[bca]
        Z3 = Q[(0, 2, 1)] + Q[(1, 0, 2)] + Q[(2, 1, 0)]  # V3[acb] + V3[bac] + V3[cba]
        Wp = P[(0, 1, 2)] + P[(2, 0, 1)] + P[(1, 2, 0)]
        Wm = P[(0, 2, 1)] + P[(1, 0, 2)] + P[(2, 1, 0)]
        d3 = eo[i] + eo[j] + eo[k] - dv
        fac = 2.0 - ((i == j) + (i == k) + (j == k))
        term = ((Y3 - 2.0 * Z3) * Wp + (Z3 - 2.0 * Y3) * Wm + 3.0 * X3) * fac / d3
        return term.sum()

    def tcorr_tjl(self):  # ccwfn.cc:795-852
        no = self.H.no
        setup = self.tuple_setup()
        ET = 0.0
        for i in range(no):
            for j in range(i + 1):
                for k in range(j + 1):
                    ET += self.tcorr_tuple(i, j, k, setup)
        return ET

    # ------------------------------------------------- (T) gradient pieces
    def N3_ijk(self, i, j, k):  # ccwfn.cc:1492-1515, numerator (the caller divides by D3)
        H, t1, t2 = self.H, self.t1, self.t2
        Voovv, fov = H.V("oovv"), H.fblk("ov")
        return (ein("ab,c->abc", Voovv[i, j], t1[k]) + ein("ac,b->abc", Voovv[i, k], t1[j])
                + ein("bc,a->abc", Voovv[j, k], t1[i]) + ein("ab,c->abc", t2[i, j], fov[k])
                + ein("ac,b->abc", t2[i, k], fov[j]) + ein("bc,a->abc", t2[j, k], fov[i]))

    def tgrad(self, ooc: bool = False):  # ccwfn.cc:1150-1316 (tgrad_ooc), :854-1142 (tgrad)
        """s1, s2 and the (T) density pieces; M3 = W3/D3 and N3 over every ordered (i,j,k).

        ooc=True follows tgrad_ooc (Doo, Dvv diagonal); ooc=False (the plugin's default,
        ugacc.cc:67) the in-core tgrad, whose stored t3 is M3 and whose l3 contracts like
        X3 + Y3, giving the full Doo and Dvv of ccwfn.cc:998-1021."""
        H, t1, t2 = self.H, self.t1, self.t2
        no, nv = H.no, H.nv
        eo, ev = np.diag(H.f)[:no], np.diag(H.f)[no:]
        Voovv, Vooov, Vvovv = H.V("oovv"), H.V("ooov"), H.V("vovv")
        dv = ev[:, None, None] + ev[None, :, None] + ev[None, None, :]
        M = np.zeros((no, no, no, nv, nv, nv))
        N = np.zeros_like(M)
        for i in range(no):
            for j in range(no):
                for k in range(no):
                    d3 = eo[i] + eo[j] + eo[k] - dv
                    M[i, j, k] = self.W3_ijk(i, j, k) / d3  # M3_ijk, ccwfn.cc:1420-1454
                    N[i, j, k] = self.N3_ijk(i, j, k) / d3

        def perm6(A, w):  # 8A(abc) - 4A(bac) - 4A(acb) - 4A(cba) + 2A(cab) + 2A(bca) over the last three axes
            o = A.ndim - 3
            T = lambda p: A.transpose(tuple(range(o)) + tuple(o + q for q in p))
            return w[0] * A - w[1] * T((1, 0, 2)) - w[1] * T((0, 2, 1)) - w[1] * T((2, 1, 0)) + w[2] * T((1, 2, 0)) \
                + w[2] * T((2, 0, 1))

        X = perm6(M, (8.0, 4.0, 2.0))
        Y = perm6(N, (8.0, 4.0, 2.0))
        # Z3[a][b][c] = 2(M[abc] - M[acb]) - (M[bac] - M[bca])
        Z = 2.0 * (M - M.transpose(0, 1, 2, 3, 5, 4)) - (M.transpose(0, 1, 2, 4, 3, 5) - M.transpose(0, 1, 2, 5, 3, 4))
        Q = 2.0 * X + Y
        s1 = np.zeros((no, nv))
        X2 = np.zeros((no, no, nv, nv))
        Doo, Dvv, Dov = np.zeros((no, no)), np.zeros((nv, nv)), np.zeros((no, nv))
        Goovv = np.zeros((no, no, nv, nv))
        Gooov = np.zeros((no, no, no, nv))
        Gvvvo = np.zeros((nv, nv, nv, no))
        for i in range(no):
            for j in range(no):
                for k in range(no):
                    m, z, q = M[i, j, k], Z[i, j, k], Q[i, j, k]
                    Dvv[np.arange(nv), np.arange(nv)] += 0.5 * ein("abc,abc->a", m, X[i, j, k] + Y[i, j, k])
                    Dov[i] += ein("abc,bc->a", m - m.transpose(2, 1, 0), 4.0 * t2[j, k] - 2.0 * t2[j, k].T)
                    s1[i] += ein("abc,bc->a", 4.0 * m - 4.0 * m.transpose(1, 0, 2) - 2.0 * m.transpose(0, 2, 1)
                                 + 2.0 * m.transpose(1, 2, 0), Voovv[j, k])
                    Goovv[i, j] += 4.0 * ein("c,abc->ab", t1[k], z)
                    X2[i] -= ein("abc,lc->lab", q, Vooov[j, k])
                    Gooov[j, i] -= ein("abc,lbc->la", q, t2[:, k])
                    X2[i, j] += ein("abc,dbc->ad", q, Vvovv[:, k])
                    Gvvvo[:, :, :, j] += ein("abc,cd->abd", q, t2[k, i])
        # second pass over (a,b,c) with occupied permutations (M3_abc/N3_abc, :1226-1250)
        Mo = M.transpose(3, 4, 5, 0, 1, 2)
        No = N.transpose(3, 4, 5, 0, 1, 2)
        Xo, Yo = perm6(Mo, (8.0, 4.0, 2.0)), perm6(No, (8.0, 4.0, 2.0))
        Doo[np.arange(no), np.arange(no)] -= 0.5 * ein("abcijk,abcijk->i", Mo, Xo + Yo)
        if not ooc:  # ccwfn.cc:999-1021
            Doo = -0.5 * ein("ilmdef,jlmdef->ij", M, X + Y)
            Dvv = 0.5 * ein("ijkbde,ijkade->ab", M, X + Y)
        s2 = X2 + X2.transpose(1, 0, 3, 2)
        self.tg = dict(s1=s1, s2=s2, Doo=Doo, Dvv=Dvv, Dov=Dov, Goovv=Goovv, Gooov=Gooov, Gvvvo=Gvvvo)
        return self.tg


# --------------------------------------------------------------------------------------
# HBAR                                                                      (hbar.cc)
# --------------------------------------------------------------------------------------
class HBAR:
    def __init__(self, H: Hamiltonian, cc: CCWfn):
        t1, t2, tau = cc.t1, cc.t2, cc.tau
        fov, V, L = H.fblk("ov"), H.V, H.L
        self.Hov = fov + ein("nf,mnef->me", t1, L("oovv"))  # :36-43
        self.Hoo = (H.fblk("oo") + ein("ie,me->mi", t1, fov) + ein("ne,mnie->mi", t1, L("ooov"))
                    + ein("inef,mnef->mi", tau, L("oovv")))  # :45-57
        self.Hvv = (H.fblk("vv") - ein("me,ma->ae", fov, t1) + ein("mf,amef->ae", t1, L("vovv"))
                    - ein("mnfa,mnfe->ae", tau, L("oovv")))  # :59-71
        self.Hoooo = V("oooo") + 2.0 * ein("je,mnie->mnij", t1, V("ooov")) + ein("ijef,mnef->mnij", tau, V("oovv"))
        self.Hvvvv = (V("vvvv") - 2.0 * ein("mb,amef->abef", t1, V("vovv"))
                      + ein("mnab,mnef->abef", tau, V("oovv")))  # :86-97
        self.Hvovv = V("vovv") - ein("na,nmef->amef", t1, V("oovv"))  # :99-107
        self.Hooov = V("ooov") + ein("if,nmef->mnie", t1, V("oovv"))  # :109-117
        self.Hovvo = (V("ovvo") + ein("jf,mbef->mbej", t1, V("ovvv")) - ein("nb,mnej->mbej", t1, V("oovo"))
                      - ein("mnef,njbf->mbej", V("oovv"), tau) + ein("njfb,mnef->mbej", t2, L("oovv")))  # :119-135
        self.Hovov = (V("ovov") + ein("jf,bmef->mbje", t1, V("vovv")) - ein("nb,mnje->mbje", t1, V("ooov"))
                      - ein("nmef,jnfb->mbje", V("oovv"), tau))  # :137-151
        Voovv = V("oovv")
        Hvvvo = V("vvvo") + ein("if,abef->abei", t1, V("vvvv"))  # :153-189
        Hvvvo -= ein("mb,amei->abei", t1, V("vovo")) + ein("ma,bmie->abei", t1, V("voov"))
        Hvvvo -= ein("imfa,mbef->abei", tau, V("ovvv")) + ein("imfb,amef->abei", tau, V("vovv"))
        Hvvvo += ein("mnab,mnei->abei", tau, V("oovo"))
        Hvvvo -= ein("me,miab->abei", fov, t2)
        Hvvvo += ein("mifb,amef->abei", t2, L("vovv"))
        Hvvvo += ein("mnef,if,mnab->abei", Voovv, t1, t2)
        Hvvvo += ein("mnef,ma,infb->abei", Voovv, t1, t2)
        Hvvvo += ein("mnef,nb,miaf->abei", Voovv, t1, t2)
        Hvvvo -= ein("mf,niab,mnfe->abei", t1, t2, L("oovv"))
        Hvvvo -= ein("na,mifb,mnfe->abei", t1, t2, L("oovv"))
        Hvvvo += ein("if,ma,nb,mnef->abei", t1, t1, t1, Voovv)
        self.Hvvvo = Hvvvo
        Hovoo = V("ovoo") + ein("je,mbie->mbij", t1, V("ovov")) + ein("ie,bmje->mbij", t1, V("voov"))  # :191-227
        Hovoo -= ein("nb,mnij->mbij", t1, V("oooo"))
        Hovoo -= ein("ineb,nmje->mbij", tau, V("ooov")) + ein("jneb,mnie->mbij", tau, V("ooov"))
        Hovoo += ein("mbef,ijef->mbij", V("ovvv"), tau)
        Hovoo += ein("me,ijeb->mbij", fov, t2)
        Hovoo += ein("mnie,njeb->mbij", L("ooov"), t2)
        Hovoo -= ein("mnef,jf,ineb->mbij", Voovv, t1, t2)
        Hovoo -= ein("mnef,ie,jnfb->mbij", Voovv, t1, t2)
        Hovoo -= ein("mnef,nb,ijef->mbij", Voovv, t1, t2)
        Hovoo += ein("ie,njfb,mnef->mbij", t1, t2, L("oovv"))
        Hovoo += ein("nf,ijeb,mnef->mbij", t1, t2, L("oovv"))
        Hovoo -= ein("jf,ie,nb,mnef->mbij", t1, t1, t1, Voovv)
        self.Hovoo = Hovoo


# --------------------------------------------------------------------------------------
# Lambda                                                                (cclambda.cc)
# --------------------------------------------------------------------------------------
class CCLambda:
    def __init__(self, cc: CCWfn, hbar: HBAR):
        self.cc, self.hb, self.H = cc, hbar, cc.H
        self.l1 = 2.0 * cc.t1  # :29-41
        self.l2 = 2.0 * (2.0 * cc.t2 - cc.t2.swapaxes(2, 3))
        self.iterations = 0
        self.iter_pseudo: list[float] = []

    def build_G(self, l2):  # :131-157
        t2 = self.cc.t2
        Goo = ein("mjab,ijab->mi", t2, l2)
        Gvv = -ein("ijeb,ijab->ae", t2, l2)
        return Goo, Gvv

    def build_l1(self, l1, l2, Goo, Gvv):  # :159-213
        hb = self.hb
        R = 2.0 * hb.Hov.copy()
        R += ein("ie,ea->ia", l1, hb.Hvv)
        R -= ein("ma,im->ia", l1, hb.Hoo)
        R += ein("me,ieam->ia", l1, 2.0 * hb.Hovvo - hb.Hovov.transpose(0, 1, 3, 2))
        R += ein("imef,efam->ia", l2, hb.Hvvvo)
        R -= ein("mnae,iemn->ia", l2, hb.Hovoo)
        R -= ein("ef,eifa->ia", Gvv, 2.0 * hb.Hvovv - hb.Hvovv.swapaxes(2, 3))
        R -= ein("mn,mina->ia", Goo, 2.0 * hb.Hooov - hb.Hooov.transpose(1, 0, 2, 3))
        tg = getattr(self.cc, "tg", None)
        if tg is not None:  # WFN=CCSD_T, DERTYPE=FIRST: :181
            R += tg["s1"]
        return R

    def build_l2(self, l1, l2, Goo, Gvv):  # :215-289
        hb, H = self.hb, self.H
        Loovv = H.L("oovv")
        Z = Loovv.copy()
        tg = getattr(self.cc, "tg", None)
        if tg is not None:  # WFN=CCSD_T, DERTYPE=FIRST: :243
            Z += 0.5 * tg["s2"]
        Z += 2.0 * ein("ia,jb->ijab", l1, hb.Hov) - ein("ja,ib->ijab", l1, hb.Hov)
        Z += ein("ijeb,ea->ijab", l2, hb.Hvv)
        Z -= ein("mjab,im->ijab", l2, hb.Hoo)
        Z += 0.5 * ein("mnab,ijmn->ijab", l2, hb.Hoooo)
        Z += 0.5 * ein("ijef,efab->ijab", l2, hb.Hvvvv)
        Z += ein("ie,ejab->ijab", l1, 2.0 * hb.Hvovv - hb.Hvovv.swapaxes(2, 3))
        Z -= ein("mb,jima->ijab", l1, 2.0 * hb.Hooov - hb.Hooov.transpose(1, 0, 2, 3))
        Z += ein("ieam,mjeb->ijab", 2.0 * hb.Hovvo - hb.Hovov.transpose(0, 1, 3, 2), l2)
        Z -= ein("jema,mibe->ijab", hb.Hovov, l2)
        Z -= ein("jeam,mieb->ijab", hb.Hovvo, l2)
        Z += ein("ae,ijeb->ijab", Gvv, Loovv)
        Z -= ein("mi,mjab->ijab", Goo, Loovv)
        return Z + Z.transpose(1, 0, 3, 2)

    def pseudoenergy(self):  # :296-311
        return 0.5 * ein("ijab,ijab->", self.H.V("oovv"), self.l2)

    def compute_lambda(self):  # :93-129
        cc = self.cc
        D1, D2 = cc.D1, cc.D2
        diis = DIIS(8)
        rms = float("inf")
        for it in range(1, cc.maxiter + 1):
            l1o, l2o = self.l1, self.l2
            Goo, Gvv = self.build_G(l2o)
            R1 = self.build_l1(l1o, l2o, Goo, Gvv)
            R2 = self.build_l2(l1o, l2o, Goo, Gvv)
            rms = math.sqrt((R1 ** 2).sum() + (R2 ** 2).sum())
            self.l1, self.l2 = l1o + R1 / D1, l2o + R2 / D2
            self.iterations = it
            if rms < cc.conv:
                break
            if cc.do_diis:
                diis.add(_pack(self.l1 - l1o, self.l2 - l2o), _pack(self.l1, self.l2))
                if diis.size() > 2:
                    self.l1, self.l2 = _unpack(diis.extrapolate(), self.l1, self.l2)
            self.iter_pseudo.append(self.pseudoenergy())
        if rms >= cc.conv:
            raise NotConverged("Computation has not converged.")


# --------------------------------------------------------------------------------------
# Densities                                                            (ccdensity.cc)
# --------------------------------------------------------------------------------------
class CCDensity:
    def __init__(self, cc: CCWfn, lam: CCLambda):
        self.cc, self.lam, self.H = cc, lam, cc.H

    def onepdm(self):  # :89-151
        t1, t2, tau = self.cc.t1, self.cc.t2, self.cc.tau
        l1, l2 = self.lam.l1, self.lam.l2
        self.Doo = -ein("ie,je->ij", t1, l1) - ein("imef,jmef->ij", t2, l2)
        self.Dvv = ein("mb,ma->ab", t1, l1) + ein("mnbe,mnae->ab", t2, l2)
        self.Dvo = l1.T.copy()
        self.Dov = 2.0 * t1 + ein("me,imae->ia", l1, 2.0 * t2 - tau.transpose(1, 0, 2, 3))
        self.Dov -= ein("mnef,ma,inef->ia", l2, t1, t2) + ein("mnef,ie,mnaf->ia", l2, t1, t2)
        tg = getattr(self.cc, "tg", None)
        if tg is not None:  # the (T) pieces the densities start from, ccdensity.cc:44-69
            self.Doo += tg["Doo"]
            self.Dvv += tg["Dvv"]
            self.Dov += tg["Dov"]
        return ein("ij,ij->", self.H.fblk("oo"), self.Doo) + ein("ab,ab->", self.H.fblk("vv"), self.Dvv)

    def twopdm(self):  # :153-339
        H = self.H
        t1, t2, tau = self.cc.t1, self.cc.t2, self.cc.tau
        l1, l2 = self.lam.l1, self.lam.l2
        V = H.V
        E = {}
        self.G = {}  # the six blocks, kept for the element-wise comparison
        Goooo = ein("ijef,klef->ijkl", tau, l2)
        E["oooo"] = 0.5 * ein("ijkl,ijkl->", V("oooo"), Goooo)
        Gvvvv = ein("mnab,mncd->abcd", tau, l2)
        E["vvvv"] = 0.5 * ein("abcd,abcd->", V("vvvv"), Gvvvv)
        self.G["Goooo"], self.G["Gvvvv"] = Goooo, Gvvvv
        # Gooov, :206-228
        G = -ein("ke,ijea->ijka", l1, 2.0 * tau - tau.swapaxes(2, 3))
        G -= ein("ie,jkae->ijka", t1, l2)
        G -= 2.0 * (ein("kmef,ja,imef->ijka", l2, t1, t2) + ein("kmef,ie,jmaf->ijka", l2, t1, t2))
        G += ein("kmef,ia,jmef->ijka", l2, t1, t2) + ein("kmef,je,imaf->ijka", l2, t1, t2)
        G += (ein("kmef,ma,ijef->ijka", l2, t1, t2) + ein("kmef,ie,mjaf->ijka", l2, t1, t2)
              + ein("kmef,jf,imea->ijka", l2, t1, t2))
        G += ein("kmef,ma,ie,jf->ijka", l2, t1, t1, t1)
        tg = getattr(self.cc, "tg", None)
        if tg is not None:
            G += tg["Gooov"]
        E["ooov"] = ein("ijka,ijka->", V("ooov"), G)
        self.G["Gooov"] = G
        # Gvvvo, :237-259
        G = ein("mc,miab->abci", l1, 2.0 * tau - tau.transpose(1, 0, 2, 3))
        G += ein("ma,imbc->abci", t1, l2)
        G += 2.0 * (ein("nmce,na,imbe->abci", l2, t1, t2) + ein("nmce,ib,nmae->abci", l2, t1, t2))
        G -= ein("nmce,nb,imae->abci", l2, t1, t2) + ein("nmce,ia,nmbe->abci", l2, t1, t2)
        G -= (ein("nmce,mb,niae->abci", l2, t1, t2) + ein("nmce,na,mibe->abci", l2, t1, t2)
              + ein("nmce,ie,nmab->abci", l2, t1, t2))
        G -= ein("nmce,mb,na,ie->abci", l2, t1, t1, t1)
        if tg is not None:
            G += tg["Gvvvo"]
        E["vvvo"] = ein("abci,abci->", V("vvvo"), G)
        self.G["Gvvvo"] = G
        # Govov, :268-276
        G = -ein("ia,jb->iajb", t1, l1)
        G -= ein("mibe,jmea->iajb", tau, l2) + ein("imbe,mjea->iajb", t2, l2)
        E["ovov"] = ein("iajb,iajb->", V("ovov"), G)
        self.G["Govov"] = G
        # Goovv, :285-328
        t2x = 2.0 * t2 - t2.swapaxes(2, 3)
        taux = 2.0 * tau - tau.swapaxes(2, 3)
        G = 4.0 * ein("ia,jb->ijab", t1, l1) + 4.0 * tau - 2.0 * tau.swapaxes(2, 3) + l2
        G += 2.0 * (2.0 * ein("me,ia,jmbe->ijab", l1, t1, t2x) - ein("me,ib,jmae->ijab", l1, t1, t2x)
                    - ein("me,ie,jmba->ijab", l1, t1, taux) - ein("me,ma,ijeb->ijab", l1, t1, t2x))
        G += 4.0 * ein("imae,mjeb->ijab", t2, l2) - 2.0 * ein("mjbe,imae->ijab", tau, l2)
        Q = 0.5 * (ein("mnef,mnab,ijef->ijab", l2, t2, t2) + ein("mnef,miae,njbf->ijab", l2, t2, t2)
                   + ein("mnef,njae,imfb->ijab", l2, t2, t2))
        Q += 2.0 * (-ein("mnef,ijae,mnbf->ijab", l2, tau, t2) - ein("mnef,imab,jnef->ijab", l2, tau, t2)
                    - ein("mnef,mjbe,inaf->ijab", l2, tau, t2) + ein("mnef,imae,jnbf->ijab", l2, t2, t2))
        Q -= (-ein("mnef,ijbe,mnaf->ijab", l2, tau, t2) - ein("mnef,imba,jnef->ijab", l2, tau, t2)
              - ein("mnef,mjae,inbf->ijab", l2, tau, t2) + ein("mnef,imbe,jnaf->ijab", l2, t2, t2))
        G += 2.0 * Q
        G += (ein("mnef,ma,nb,ijef->ijab", l2, t1, t1, t2) + ein("mnef,ie,jf,mnab->ijab", l2, t1, t1, t2)
              + ein("mnef,ma,ie,njbf->ijab", l2, t1, t1, t2) + ein("mnef,nb,jf,miae->ijab", l2, t1, t1, t2)
              + ein("mnef,na,je,imfb->ijab", l2, t1, t1, t2) + ein("mnef,if,mb,njae->ijab", l2, t1, t1, t2))
        G += ein("mnef,ma,nb,ie,jf->ijab", l2, t1, t1, t1, t1)
        if tg is not None:
            G += tg["Goovv"]
        E["oovv"] = 0.5 * ein("ijab,ijab->", V("oovv"), G)
        self.G["Goovv"] = G
        self.E2 = E
        return sum(E.values())


# --------------------------------------------------------------------------------------
# Perturbed wavefunctions                                                 (ccpert.cc)
# --------------------------------------------------------------------------------------
class CCPert:
    def __init__(self, pert: np.ndarray, omega: float, cc: CCWfn, hbar: HBAR, lam: CCLambda):
        self.pert, self.omega, self.cc, self.hb, self.lam, self.H = pert, omega, cc, hbar, lam, cc.H
        no = cc.H.no
        self.pov, self.poo, self.pvv, self.pvo = pert[:no, no:], pert[:no, :no], pert[no:, no:], pert[no:, :no]
        self.pertbar()
        hoo, hvv = np.diag(hbar.Hoo), np.diag(hbar.Hvv)  # :39-50
        self.D1 = hoo[:, None] - hvv[None, :]
        self.D2 = hoo[:, None, None, None] + hoo[None, :, None, None] - hvv[None, None, :, None] - hvv[None, None, None, :]
        self.X1 = self.Avo.T / (self.D1 + omega)  # :57-73
        Ax = self.Avvoo.transpose(2, 3, 0, 1) + self.Avvoo.transpose(3, 2, 1, 0)
        self.X2 = Ax / (self.D2 + omega)
        self.Y1 = self.X1.copy()
        self.Y2 = self.X2.copy()
        self.iterations = {"right": 0, "left": 0}

    def pertbar(self):  # :109-175
        t1, t2 = self.cc.t1, self.cc.t2
        pov = self.pov
        self.Aov = pov.copy()
        self.Aoo = self.poo + ein("ie,me->mi", t1, pov)
        self.Avv = self.pvv - ein("ma,me->ae", t1, pov)
        self.Avo = (self.pvo + ein("ie,ae->ai", t1, self.pvv) - ein("ma,mi->ai", t1, self.poo)
                    + ein("miea,me->ai", 2.0 * t2 - t2.transpose(1, 0, 2, 3), pov)
                    - ein("ie,ma,me->ai", t1, t1, pov))
        self.Aovoo = ein("ijeb,me->mbij", t2, pov)
        self.Avvvo = -ein("miab,me->abei", t2, pov)
        self.Avvoo = ein("ijeb,ae->abij", t2, self.Avv) - ein("mjab,mi->abij", t2, self.Aoo)

    def pseudoresponse(self, hand):  # :233-253
        X1, X2 = (self.X1, self.X2) if hand == "right" else (self.Y1, self.Y2)
        p1 = 2.0 * ein("ia,ai->", X1, self.Avo)
        p2 = 2.0 * ein("ijab,abij->", 2.0 * X2 - X2.swapaxes(2, 3), self.Avvoo)
        return -2.0 * (p1 + p2)

    def build_X(self, X1o, X2o):  # :373-473
        hb, H, w = self.hb, self.H, self.omega
        t2 = self.cc.t2
        R1 = self.Avo.T - w * X1o
        R1 += ein("ie,ae->ia", X1o, hb.Hvv)
        R1 -= ein("ma,mi->ia", X1o, hb.Hoo)
        R1 += ein("me,maei->ia", X1o, 2.0 * hb.Hovvo - hb.Hovov.transpose(0, 1, 3, 2))
        R1 += ein("me,miea->ia", hb.Hov, 2.0 * X2o - X2o.transpose(1, 0, 2, 3))
        R1 += ein("imef,amef->ia", X2o, 2.0 * hb.Hvovv - hb.Hvovv.swapaxes(2, 3))
        R1 -= ein("mnae,mnie->ia", X2o, 2.0 * hb.Hooov - hb.Hooov.transpose(1, 0, 2, 3))
        Lv = H.L("oovv")
        Zvv = ein("amef,mf->ae", 2.0 * hb.Hvovv - hb.Hvovv.swapaxes(2, 3), X1o) - ein("mnef,mnaf->ae", Lv, X2o)
        Zoo = -ein("mnie,ne->mi", 2.0 * hb.Hooov - hb.Hooov.transpose(1, 0, 2, 3), X1o) - ein("mnef,inef->mi", Lv, X2o)
        R2 = self.Avvoo.transpose(2, 3, 0, 1) - 0.5 * w * X2o
        R2 += ein("ie,abej->ijab", X1o, hb.Hvvvo)
        R2 -= ein("ma,mbij->ijab", X1o, hb.Hovoo)
        R2 += ein("mi,mjab->ijab", Zoo, t2)
        R2 += ein("ae,ijeb->ijab", Zvv, t2)
        R2 += ein("ijeb,ae->ijab", X2o, hb.Hvv)
        R2 -= ein("mjab,mi->ijab", X2o, hb.Hoo)
        R2 += 0.5 * ein("mnab,mnij->ijab", X2o, hb.Hoooo)
        R2 += 0.5 * ein("ijef,abef->ijab", X2o, hb.Hvvvv)
        R2 -= ein("imeb,maje->ijab", X2o, hb.Hovov) + ein("imea,mbej->ijab", X2o, hb.Hovvo)
        R2 += ein("miea,mbej->ijab", X2o, 2.0 * hb.Hovvo - hb.Hovov.transpose(0, 1, 3, 2))
        return R1, R2 + R2.transpose(1, 0, 3, 2)

    def build_G(self, Y2o):  # :500-527
        t2 = self.cc.t2
        return ein("mjab,ijab->mi", t2, Y2o), -ein("ijeb,ijab->ae", t2, Y2o)

    def build_Y(self, Y1o, Y2o):  # :530-881
        hb, H, w = self.hb, self.H, self.omega
        t2 = self.cc.t2
        l1, l2 = self.lam.l1, self.lam.l2
        X1, X2 = self.X1, self.X2
        Lovvv = None
        Goo, Gvv = self.build_G(Y2o)
        Hovvo_x = 2.0 * hb.Hovvo - hb.Hovov.transpose(0, 1, 3, 2)   # [i,e,a,m]
        Hvovv_x = 2.0 * hb.Hvovv - hb.Hvovv.swapaxes(2, 3)          # 2H[e,i,f,a]-H[e,i,a,f]
        Hooov_x = 2.0 * hb.Hooov - hb.Hooov.transpose(1, 0, 2, 3)   # 2H[m,i,n,a]-H[i,m,n,a]
        Loovv = H.L("oovv")
        # ----- Y1, build_Y1 :530-728
        R1 = 2.0 * self.pov + w * Y1o
        R1 += ein("ie,ea->ia", Y1o, hb.Hvv)
        R1 -= ein("ma,im->ia", Y1o, hb.Hoo)
        R1 += ein("me,ieam->ia", Y1o, Hovvo_x)
        R1 += ein("imef,efam->ia", Y2o, hb.Hvvvo)
        R1 -= ein("mnae,iemn->ia", Y2o, hb.Hovoo)
        R1 -= ein("ef,eifa->ia", Gvv, Hvovv_x)
        R1 -= ein("mn,mina->ia", Goo, Hooov_x)
        R1 += 2.0 * ein("me,imae->ia", X1, Loovv)                                   # (i)
        R1 -= ein("ma,im->ia", l1, self.Aoo)                                         # (m)
        R1 += ein("ie,ea->ia", l1, self.Avv)                                         # (m)
        R1 += ein("imfe,feam->ia", l2, self.Avvvo)                                   # (n)
        R1 -= 0.5 * ein("mnea,ienm->ia", l2, self.Aovoo)                             # (n)
        R1 -= 0.5 * ein("mnae,iemn->ia", l2, self.Aovoo)                             # (n)
        R1 -= ein("me,ma,ie->ia", X1, hb.Hov, l1)                                    # (q)
        R1 -= ein("me,ie,ma->ia", X1, hb.Hov, l1)
        R1 -= ein("me,mina,ne->ia", X1, Hooov_x, l1)
        R1 -= ein("me,imne,na->ia", X1, Hooov_x, l1)
        R1 += ein("me,fmae,if->ia", X1, Hvovv_x, l1)
        R1 += ein("me,fiea,mf->ia", X1, Hvovv_x, l1)
        R1 += 2.0 * ein("mnef,imae,nf->ia", X2, Loovv, l1)                           # (r)
        R1 -= ein("mnef,imaf,ne->ia", X2, Loovv, l1)
        R1 -= ein("mnef,mief,na->ia", X2, Loovv, l1)
        R1 -= ein("mnef,nmfa,ie->ia", X2, Loovv, l1)
        R1 -= ein("me,mfna,nief->ia", X1, hb.Hovov, l2)                              # (s)
        R1 -= ein("me,ifne,nmaf->ia", X1, hb.Hovov, l2)
        R1 -= ein("me,mfan,nife->ia", X1, hb.Hovvo, l2)
        R1 -= ein("me,ifen,nmfa->ia", X1, hb.Hovvo, l2)
        R1 += 0.5 * ein("me,fgae,imfg->ia", X1, hb.Hvvvv, l2)
        R1 += 0.5 * ein("me,fgea,mifg->ia", X1, hb.Hvvvv, l2)
        R1 += 0.5 * ein("me,imno,noae->ia", X1, hb.Hoooo, l2)
        R1 += 0.5 * ein("me,mino,noea->ia", X1, hb.Hoooo, l2)
        R1 -= ein("inaf,nb,jmfe,jmbe->ia", Loovv, X1, t2, l2)                        # three-body
        R1 -= ein("mief,me,jnfb,jnab->ia", Loovv, X1, t2, l2)
        R1 -= ein("mnea,me,jnfb,jifb->ia", Loovv, X1, t2, l2)
        R1 -= ein("inaf,jf,nmeb,jmeb->ia", Loovv, X1, t2, l2)
        R1 -= ein("mnef,ma,nife->ia", X2, hb.Hov, l2)                                # (t)
        R1 -= ein("mnef,ie,nmfa->ia", X2, hb.Hov, l2)
        R1 -= ein("mnef,gnea,imfg->ia", X2, hb.Hvovv, l2)
        R1 -= ein("mnef,gnae,mifg->ia", X2, hb.Hvovv, l2)
        R1 -= ein("mnef,gief,nmag->ia", X2, hb.Hvovv, l2)
        R1 += ein("mnef,gmae,nifg->ia", X2, Hvovv_x, l2)
        R1 += ein("mnef,giea,nmfg->ia", X2, Hvovv_x, l2)
        R1 += ein("mnef,mnoa,oief->ia", X2, hb.Hooov, l2)
        R1 += ein("mnef,inoe,omaf->ia", X2, hb.Hooov, l2)
        R1 += ein("mnef,miof,onea->ia", X2, hb.Hooov, l2)
        R1 -= ein("mnef,mioa,nofe->ia", X2, Hooov_x, l2)
        R1 -= ein("mnef,imoe,nofa->ia", X2, Hooov_x, l2)
        # ----- Y2, build_Y2 :730-881
        V = H.V
        R2 = 0.5 * w * Y2o
        R2 += 2.0 * ein("ia,jb->ijab", Y1o, hb.Hov) - ein("ja,ib->ijab", Y1o, hb.Hov)
        R2 += ein("ijeb,ea->ijab", Y2o, hb.Hvv)
        R2 -= ein("mjab,im->ijab", Y2o, hb.Hoo)
        R2 += 0.5 * ein("mnab,ijmn->ijab", Y2o, hb.Hoooo)
        R2 += 0.5 * ein("ijef,efab->ijab", Y2o, hb.Hvvvv)
        R2 += ein("ie,ejab->ijab", Y1o, Hvovv_x)
        R2 -= ein("mb,jima->ijab", Y1o, Hooov_x)
        R2 += ein("mjeb,ieam->ijab", Y2o, Hovvo_x)
        R2 -= ein("mibe,jema->ijab", Y2o, hb.Hovov)
        R2 -= ein("mieb,jeam->ijab", Y2o, hb.Hovvo)
        R2 += ein("ae,ijeb->ijab", Gvv, Loovv)
        R2 -= ein("mi,mjab->ijab", Goo, Loovv)
        R2 += 2.0 * ein("jb,ia->ijab", l1, self.pov) - ein("ib,ja->ijab", l1, self.pov)   # (o)
        R2 += ein("ijeb,ea->ijab", l2, self.Avv)                                           # (p)
        R2 -= ein("mjab,im->ijab", l2, self.Aoo)
        R2 -= ein("me,ja,mieb->ijab", X1, l1, Loovv)                                       # (u)
        R2 -= ein("me,mb,ijae->ijab", X1, l1, Loovv)
        R2 -= ein("me,ie,jmba->ijab", X1, l1, Loovv)
        R2 += 2.0 * ein("me,jb,imae->ijab", X1, l1, Loovv)
        R2 -= ein("ma,jibe,me->ijab", hb.Hov, l2, X1)                                      # (w)
        R2 -= ein("ie,jmba,me->ijab", hb.Hov, l2, X1)
        R2 -= ein("fmba,jife,me->ijab", hb.Hvovv, l2, X1)
        R2 -= ein("fjea,mifb,me->ijab", hb.Hvovv, l2, X1)
        R2 -= ein("fibe,jmfa,me->ijab", hb.Hvovv, l2, X1)
        R2 += ein("fmae,jibf,me->ijab", Hvovv_x, l2, X1)
        R2 += ein("fiea,jmbf,me->ijab", Hvovv_x, l2, X1)
        R2 += ein("jmna,nibe,me->ijab", hb.Hooov, l2, X1)
        R2 += ein("mjna,nieb,me->ijab", hb.Hooov, l2, X1)
        R2 += ein("jine,nmba,me->ijab", hb.Hooov, l2, X1)
        R2 -= ein("mina,jnbe,me->ijab", Hooov_x, l2, X1)
        R2 -= ein("imne,jnba,me->ijab", Hooov_x, l2, X1)
        Voovv = V("oovv")
        R2 += 0.25 * ein("nmab,jief,mnef->ijab", Voovv, l2, X2)                            # (x)
        R2 += 0.25 * ein("mnab,jife,mnef->ijab", Voovv, l2, X2)
        R2 += 0.25 * ein("jnae,mifb,mnef->ijab", Voovv, l2, X2)
        R2 += 0.25 * ein("jmaf,nieb,mnef->ijab", Voovv, l2, X2)
        R2 += 0.25 * ein("njae,mibf,mnef->ijab", Voovv, l2, X2)
        R2 += 0.25 * ein("mjaf,nibe,mnef->ijab", Voovv, l2, X2)
        R2 += 0.25 * ein("jnea,imfb,mnef->ijab", Voovv, l2, X2)
        R2 += 0.25 * ein("jmfa,ineb,mnef->ijab", Voovv, l2, X2)
        R2 += 0.25 * ein("njea,imbf,mnef->ijab", Voovv, l2, X2)
        R2 += 0.25 * ein("mjfa,inbe,mnef->ijab", Voovv, l2, X2)
        R2 += 0.25 * ein("jief,nmab,mnef->ijab", Voovv, l2, X2)
        R2 += 0.25 * ein("jife,mnab,mnef->ijab", Voovv, l2, X2)
        R2 -= 0.5 * ein("imaf,jnbe,mnef->ijab", Loovv, l2, X2)
        R2 -= 0.5 * ein("inae,jmbf,mnef->ijab", Loovv, l2, X2)
        R2 -= 0.5 * ein("mief,jnba,mnef->ijab", Loovv, l2, X2)
        R2 -= 0.5 * ein("mnea,jibf,mnef->ijab", Loovv, l2, X2)
        R2 -= 0.5 * ein("nmfa,jibe,mnef->ijab", Loovv, l2, X2)
        R2 -= 0.5 * ein("nife,jmba,mnef->ijab", Loovv, l2, X2)
        R2 -= ein("ijae,nmfb,mnef->ijab", Loovv, l2, X2)
        R2 -= ein("imab,njfe,mnef->ijab", Loovv, l2, X2)
        R2 -= ein("mjea,nifb,mnef->ijab", Loovv, l2, X2)
        R2 += 2.0 * ein("imae,njfb,mnef->ijab", Loovv, l2, X2)
        del Lovvv
        return R1, R2 + R2.transpose(1, 0, 3, 2)

    def solve(self, hand: str):  # :177-229
        cc = self.cc
        w = self.omega
        diis = DIIS(8)
        rms = float("inf")
        for it in range(1, cc.maxiter + 1):
            if hand == "right":
                o1, o2 = self.X1, self.X2
                R1, R2 = self.build_X(o1, o2)
            else:
                o1, o2 = self.Y1, self.Y2
                R1, R2 = self.build_Y(o1, o2)
            rms = math.sqrt((R1 ** 2).sum() + (R2 ** 2).sum())  # :346-371
            n1, n2 = o1 + R1 / (self.D1 + w), o2 + R2 / (self.D2 + w)
            self.iterations[hand] = it
            if rms < cc.conv:
                self._set(hand, n1, n2)
                break
            if cc.do_diis:
                diis.add(_pack(n1 - o1, n2 - o2), _pack(n1, n2))
                if diis.size() > 2:
                    n1, n2 = _unpack(diis.extrapolate(), n1, n2)
            self._set(hand, n1, n2)
        if rms >= cc.conv:
            raise NotConverged("Computation has not converged.")

    def _set(self, hand, a1, a2):
        if hand == "right":
            self.X1, self.X2 = a1, a2
        else:
            self.Y1, self.Y2 = a1, a2


def linresp(X: CCPert, Y: CCPert) -> float:  # ccresp.cc:28-124
    l1, l2 = X.lam.l1, X.lam.l2
    Ax = X.Avvoo.transpose(2, 3, 0, 1) + X.Avvoo.transpose(3, 2, 1, 0)  # [i,j,a,b]
    polar1 = ein("ai,ia->", X.Avo, Y.Y1) + 0.5 * ein("ijab,ijab->", Ax, Y.Y2)
    p = ein("ia,jb,ijab->", l1, X.pov, 2.0 * Y.X2 - Y.X2.swapaxes(2, 3))
    p += ein("ia,ac,ic->", l1, X.Avv, Y.X1)
    p -= ein("ia,ki,ka->", l1, X.Aoo, Y.X1)
    p += ein("ijbc,ia,bcaj->", l2, Y.X1, X.Avvvo)
    p -= 0.5 * ein("ijab,ka,kbij->", l2, Y.X1, X.Aovoo)
    p -= 0.5 * ein("ijab,kb,kaji->", l2, Y.X1, X.Aovoo)
    p -= 0.5 * ein("ijab,kjab,ki->", l2, Y.X2, X.Aoo)
    p -= 0.5 * ein("ijab,kiba,kj->", l2, Y.X2, X.Aoo)
    p += 0.5 * ein("ijab,ijac,bc->", l2, Y.X2, X.Avv)
    p += 0.5 * ein("ijab,jibc,ac->", l2, Y.X2, X.Avv)
    p += 2.0 * ein("ia,ia->", X.pov, Y.X1)
    return -(polar1 + p)


def response(cc: CCWfn, hbar: HBAR, lam: CCLambda, perts, omega: float, hand: str = "right"):
    """The recipe of ugacc.cc:158-227: Mu/L perturbed wavefunctions per axis, the
    symmetrised dipole polarizability and the length-gauge optical rotation tensor."""
    P = {}
    axes = "XYZ"
    for x in range(3):
        P["Mu" + axes[x]] = CCPert(perts[x], omega, cc, hbar, lam)
        P["Mu" + axes[x]].solve("right")
        P["L" + axes[x]] = CCPert(perts[3 + x], omega, cc, hbar, lam)
        P["L" + axes[x]].solve("right")
        if hand == "left":
            P["Mu" + axes[x]].solve("left")
            P["L" + axes[x]].solve("left")
    alpha, rot = {}, {}
    for p in range(3):
        for q in range(p + 1):
            A, B = P["Mu" + axes[p]], P["Mu" + axes[q]]
            v = linresp(A, B) if p == q else 0.5 * linresp(A, B) + 0.5 * linresp(B, A)
            alpha[axes[p] + axes[q]] = v
    for p in range(3):
        for q in range(3):
            A, B = P["Mu" + axes[p]], P["L" + axes[q]]
            rot[axes[p] + axes[q]] = -(0.5 * linresp(A, B) - 0.5 * linresp(B, A))
    return alpha, rot, P
