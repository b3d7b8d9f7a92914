"""Test infrastructure: NOT part of the product.

Pure-Python restatement of the reference's model-space bookkeeping, used by the
tests and by the golden-fixture script to lay out and generate operators
independently of the product's C++ host code:

* orbit order            -- ModelSpace::Init, src/ModelSpace.cc:369-401
                            (N ascending, l = N, N-2, ..., j2 = 2l+1 then 2l-1,
                            tz2 = -1 then +1; index = order of AddOrbit,
                            src/ModelSpace.cc:923-933)
* reference occupations  -- ModelSpace::GetOrbitsAZ, src/ModelSpace.cc:610-645
* kets |pq>, p <= q      -- ModelSpace::SetupKets / Index2, src/ModelSpace.cc:1108-1160
* pp / hh / ph classes   -- src/ModelSpace.cc:1150-1165 (OCC_CUT = 1e-6, :14)
* 2b channels            -- ch = 6J + 2(Tz+1) + parity (src/ModelSpace.cc:1046-1053),
                            TwoBodyChannel::CheckChannel_ket (src/TwoBodyChannel.cc:142-151),
                            nTwoBodyChannels = 6 (j2max + 1) (src/ModelSpace.cc:936-946)
* cross-coupled channels -- TwoBodyChannel_CC::CheckChannel_ket (src/TwoBodyChannel.cc:180-188)

It also defines the operator "arena" (flat FP64 array) shared by the product,
the C oracle and the reference harness: ZeroBody at [0], OneBody N x N
column-major at [32], then one n x n column-major block per two-body channel in
channel-index order, each block starting on a multiple of 32 doubles.
"""

import numpy as np

OCC_CUT = 1e-6


def _round32(x):
    return (x + 31) // 32 * 32


def reference_occupations(orbits, A, Z):
    """Filling of GetOrbitsAZ (src/ModelSpace.cc:610-645): shells in order of
    N, and within N the order g = 2N+1, 2N-3, ... (|g| = j2, sign -> l)."""
    emax = max(2 * o[0] + o[1] for o in orbits)
    occ = {}
    zz = 0.0
    nn = 0.0
    for N in range(emax + 1):
        for g in range(2 * N + 1, -2 * N - 1, -4):
            j2 = abs(g)
            l = (j2 + 1) // 2 if g < 0 else (j2 - 1) // 2
            n = (N - l) // 2
            if zz < Z:
                dz = min(Z - zz, j2 + 1.0)
                occ[(n, l, j2, -1)] = dz / (j2 + 1.0)
                zz += dz
            if nn < A - Z:
                dn = min(A - Z - nn, j2 + 1.0)
                occ[(n, l, j2, 1)] = dn / (j2 + 1.0)
                nn += dn
            if zz == Z and nn == A - Z:
                return occ
    raise ValueError("model space too small for A=%g Z=%g" % (A, Z))


class RefModelSpace:
    """Channel bookkeeping of ModelSpace(emax, reference, reference)."""

    def __init__(self, emax, A=16, Z=8):
        self.emax = emax
        orbits = []
        for N in range(emax + 1):
            for l in range(N, -1, -2):
                n = (N - l) // 2
                for j2 in (2 * l + 1, 2 * l - 1):
                    if j2 <= 0:
                        continue
                    for tz in (-1, 1):
                        orbits.append((n, l, j2, tz))
        occmap = reference_occupations(orbits, A, Z)
        self.orbits = orbits
        self.norb = len(orbits)
        self.n = np.array([o[0] for o in orbits])
        self.l = np.array([o[1] for o in orbits])
        self.j2 = np.array([o[2] for o in orbits])
        self.tz2 = np.array([o[3] for o in orbits])
        self.occ = np.array([occmap.get(o, 0.0) for o in orbits])
        self.holes = [i for i in range(self.norb) if self.occ[i] >= OCC_CUT]
        self.j2max = int(self.j2.max())
        self.nch = 6 * (self.j2max + 1)
        kets = [(p, q) for p in range(self.norb) for q in range(p, self.norb)]
        self.kets = kets
        self.channels = []
        self.cc_channels = []
        for ch in range(self.nch):
            J = ch // 6
            Tz = (ch % 6) // 2 - 1
            par = ch % 2
            lst = []
            lst_cc = []
            for (p, q) in kets:
                jp, jq = self.j2[p], self.j2[q]
                if (self.l[p] + self.l[q]) % 2 != par:
                    continue
                if jp + jq < 2 * J or abs(jp - jq) > 2 * J:
                    continue
                if (self.tz2[p] + self.tz2[q]) == 2 * Tz and not (p == q and J % 2 == 1):
                    lst.append((p, q))
                if abs(self.tz2[p] - self.tz2[q]) == 2 * Tz:
                    lst_cc.append((p, q))
            self.channels.append((J, par, Tz, lst))
            self.cc_channels.append((J, par, Tz, lst_cc))
        # arena layout
        cur = _round32(32 + self.norb * self.norb)
        self.off2 = []
        for ch in range(self.nch):
            n = len(self.channels[ch][3])
            self.off2.append(cur)
            cur = _round32(cur + n * n)
        self.arena_size = cur

    def ket_class(self, p, q):
        hp = self.occ[p] > OCC_CUT
        hq = self.occ[q] > OCC_CUT
        if hp and hq:
            return "hh"
        if hp != hq:
            return "ph"
        return "pp"

    def onebody_channels(self):
        """Orbits grouped by (l, j2, tz2): the one-body channels of a scalar
        operator (Operator::SetUpOneBodyChannels, src/Operator.cc:248-291)."""
        groups = {}
        for i in range(self.norb):
            groups.setdefault((int(self.l[i]), int(self.j2[i]), int(self.tz2[i])), []).append(i)
        return list(groups.values())

    # ---- arena views -------------------------------------------------------
    def onebody(self, arena):
        N = self.norb
        return arena[32:32 + N * N].reshape(N, N, order="F")

    def block(self, arena, ch):
        n = len(self.channels[ch][3])
        o = self.off2[ch]
        return arena[o:o + n * n].reshape(n, n, order="F")

    def random_operator(self, seed, hermitian=True):
        """Seeded random operator: uniform[-1,1] entries on symmetry-allowed
        elements, (anti)symmetrised, each 2b channel block and the 1b matrix
        scaled to unit Frobenius norm."""
        rng = np.random.Generator(np.random.PCG64(seed))
        a = np.zeros(self.arena_size)
        sgn = 1.0 if hermitian else -1.0
        a[0] = rng.uniform(-1, 1) if hermitian else 0.0
        one = self.onebody(a)
        for grp in self.onebody_channels():
            m = len(grp)
            R = rng.uniform(-1, 1, size=(m, m))
            S = 0.5 * (R + sgn * R.T)
            one[np.ix_(grp, grp)] = S
        nrm = np.linalg.norm(one)
        if nrm > 0:
            one /= nrm
        for ch in range(self.nch):
            n = len(self.channels[ch][3])
            if n == 0:
                continue
            R = rng.uniform(-1, 1, size=(n, n))
            S = 0.5 * (R + sgn * R.T)
            f = np.linalg.norm(S)
            if f > 0:
                S /= f
            self.block(a, ch)[:, :] = S
        return a

    def flow_hamiltonian(self, seed, v2=1.0):
        """Seeded Hamiltonian for a synthetic Magnus flow: one-body diagonal
        2n+l+3/2 (oscillator energies in units of hbar*omega), symmetric
        off-diagonal part uniform[-0.1,0.1] within each (l, j2, tz2) block,
        two-body part a random hermitian operator (as random_operator) with
        every channel block scaled to Frobenius norm v2, ZeroBody 0."""
        a = self.random_operator(seed, hermitian=True)
        rng = np.random.Generator(np.random.PCG64(seed + 7919))
        a[0] = 0.0
        one = self.onebody(a)
        one[:, :] = 0.0
        for grp in self.onebody_channels():
            m = len(grp)
            R = rng.uniform(-0.1, 0.1, size=(m, m))
            S = np.triu(R, 1)
            S = S + S.T
            S[np.diag_indices(m)] = [2 * self.n[i] + self.l[i] + 1.5 for i in grp]
            one[np.ix_(grp, grp)] = S
        a[self.off2[0]:] *= v2
        return a

    # ---- tensor operators (rank_J = lam, rank_T = trank, parity) -------------
    def tensor_blocks(self, lam, trank, parity):
        """Two-body blocks of a tensor operator in TwoBodyME::Allocate order
        (src/TwoBodyME.cc:77-95): (ch_bra, ch_ket), ch_bra <= ch_ket, with
        |J_bra - J_ket| <= lam <= J_bra + J_ket, |Tz_bra - Tz_ket| = trank and
        parity_bra + parity_ket + parity even."""
        out = []
        for cb in range(self.nch):
            Jb, pb, Tb, _ = self.channels[cb]
            for ck in range(cb, self.nch):
                Jk, pk, Tk, _ = self.channels[ck]
                if abs(Jb - Jk) > lam or Jb + Jk < lam:
                    continue
                if abs(Tb - Tk) != trank:
                    continue
                if (pb + pk + parity) % 2:
                    continue
                out.append((cb, ck))
        return out

    def tensor_layout(self, lam, trank, parity):
        """Arena of a tensor operator: ZeroBody at [0], OneBody N x N at [32],
        then every block of tensor_blocks (n_bra x n_ket, column-major), each
        starting on a multiple of 32 doubles.  Returns (blocks, offsets, size)."""
        blocks = self.tensor_blocks(lam, trank, parity)
        cur = _round32(32 + self.norb * self.norb)
        offs = []
        for cb, ck in blocks:
            offs.append(cur)
            cur = _round32(cur + len(self.channels[cb][3]) * len(self.channels[ck][3]))
        return blocks, offs, cur

    def tensor_onebody_allowed(self, i, j, lam, trank, parity):
        """<i||T||j> allowed by Operator::SetUpOneBodyChannels (src/Operator.cc:248-291)."""
        if (self.l[i] + self.l[j] + parity) % 2:
            return False
        if abs(self.j2[i] - self.j2[j]) > 2 * lam or self.j2[i] + self.j2[j] < 2 * lam:
            return False
        return abs(self.tz2[i] - self.tz2[j]) == 2 * trank

    def random_tensor(self, seed, lam, trank, parity, hermitian=True):
        """Seeded random reduced tensor operator in the tensor_layout arena:
        uniform[-1,1] on allowed elements; one-body <j||T||i> = h (-1)^(ji-jj)
        <i||T||j> (the reduced-element conjugation of Operator's one-body part);
        diagonal two-body blocks (ch, ch) symmetric (h = 1) or antisymmetric;
        every block and the one-body matrix scaled to unit Frobenius norm."""
        rng = np.random.Generator(np.random.PCG64(seed))
        blocks, offs, size = self.tensor_layout(lam, trank, parity)
        a = np.zeros(size)
        h = 1.0 if hermitian else -1.0
        N = self.norb
        one = a[32:32 + N * N].reshape(N, N, order="F")
        for i in range(N):
            for j in range(i, N):
                if not self.tensor_onebody_allowed(i, j, lam, trank, parity):
                    continue
                ph = -1.0 if ((self.j2[i] - self.j2[j]) // 2) % 2 else 1.0
                if i == j and h * ph < 0:
                    continue
                v = rng.uniform(-1, 1)
                one[i, j] = v
                one[j, i] = h * ph * v
        nrm = np.linalg.norm(one)
        if nrm > 0:
            one /= nrm
        for (cb, ck), o in zip(blocks, offs):
            nb, nk = len(self.channels[cb][3]), len(self.channels[ck][3])
            if nb == 0 or nk == 0:
                continue
            R = rng.uniform(-1, 1, size=(nb, nk))
            if cb == ck:
                R = 0.5 * (R + h * R.T)
            f = np.linalg.norm(R)
            if f > 0:
                R /= f
            a[o:o + nb * nk] = R.ravel(order="F")
        return a

    def norm(self, arena):
        """Operator::Norm for a scalar operator (src/Operator.cc:1610-1651,
        src/TwoBodyME.cc:703-723)."""
        one = self.onebody(arena)
        n1 = float(np.sum(one * one * (self.j2[:, None] + 1)))
        n2 = 0.0
        for ch in range(self.nch):
            if len(self.channels[ch][3]) == 0:
                continue
            J = self.channels[ch][0]
            f = np.linalg.norm(self.block(arena, ch)) * (2 * J + 1)
            n2 += f * f
        return float(np.sqrt(n1 + n2))


def read_ref_tables(path):
    """Parse the tables.txt written by oracle/ref_harness.cc."""
    with open(path) as f:
        toks = f.read().split("\n")
    it = iter(toks)
    out = {"orbits": [], "channels": [], "cc_channels": []}
    hdr = next(it).split()
    for _ in range(int(hdr[1])):
        v = next(it).split()
        out["orbits"].append((int(v[1]), int(v[2]), int(v[3]), int(v[4]), float(v[5])))
    hdr = next(it).split()
    for _ in range(int(hdr[1])):
        v = list(map(int, next(it).split()))
        kets = [(v[5 + 2 * i], v[6 + 2 * i]) for i in range(v[4])]
        cls = {}
        for _k in range(3):
            w = next(it).split()
            cls[w[0]] = list(map(int, w[2:]))
        out["channels"].append((v[1], v[2], v[3], kets, cls))
    hdr = next(it).split()
    for _ in range(int(hdr[1])):
        v = list(map(int, next(it).split()))
        kets = [(v[5 + 2 * i], v[6 + 2 * i]) for i in range(v[4])]
        cls = {}
        for _k in range(2):
            w = next(it).split()
            cls[w[0]] = list(map(int, w[2:]))
        out["cc_channels"].append((v[1], v[2], v[3], kets, cls))
    return out
