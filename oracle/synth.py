"""Seeded synthetic water trajectories in numpy -- TEST/BENCH INFRASTRUCTURE ONLY.

A restatement of the project's frame generator (calcir_gb300/csrc/host_synth.cpp) that
loads no compiled code of this repository, so that bench.py's reference arm times the
reference algorithm on the same frames as the GPU job without touching libcalcir.so.
Only tests/ and bench.py's CPU legs may import it.

Model (as the generator states it): rigid TIP4P/2005 water (O-H 0.09572 nm, HOH 104.52 deg,
M 0.01546 nm along the bisector), atoms O, H1, H2, M per molecule.  Frame 0 puts O on a
jittered simple-cubic lattice with uniformly random orientations; every later frame moves
each molecule in turn by a Gaussian translation and a rotation about a random axis,
redrawing (up to max_tries times) any move that brings an O or H within min_contact of
another molecule's O or H, against the molecules as they stand at that moment (earlier
molecules already moved).  Random numbers are a splitmix-style hash of (seed, frame,
molecule, attempt, draw); Gaussians are Irwin-Hall sums of 12 uniforms.

The arithmetic follows the generator's order of operations in IEEE double precision with
no fused multiply-adds, so the frames are bit-identical (tests/test_synth_port.py checks
this against the library).  Molecules are processed in vectorised passes: all proposals
of a frame are drawn at once, and the sequential accept/reject order is restored exactly
by re-checking from the first molecule whose outcome changes.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)
_GOLD = np.uint64(0x9E3779B97F4A7C15)
_C1 = np.uint64(0xBF58476D1CE4E5B9)
_C2 = np.uint64(0x94D049BB133111EB)
_SALT = np.uint64(0x5851F42D4C957F2D)
_STEP = np.uint64(0xD1B54A32D192ED03)

R_OH = 0.09572
SIN_HALF = 0.790796413773152
COS_HALF = 0.6120792693463173
D_OM = 0.01546
BODY = np.array([[0.0, 0.0, 0.0],
                 [R_OH * SIN_HALF, 0.0, R_OH * COS_HALF],
                 [-R_OH * SIN_HALF, 0.0, R_OH * COS_HALF],
                 [0.0, 0.0, D_OM]])


def _mix64(x):
    with np.errstate(over="ignore"):
        x = np.asarray(x, np.uint64) + _GOLD
        x = (x ^ (x >> np.uint64(30))) * _C1
        x = (x ^ (x >> np.uint64(27))) * _C2
        return x ^ (x >> np.uint64(31))


class Streams:
    """One random stream per molecule (vectorised over molecules)."""

    def __init__(self, seed, frame, mols, attempts):
        mols = np.asarray(mols, np.uint64)
        att = np.broadcast_to(np.asarray(attempts, np.uint64), mols.shape)
        self.base = _mix64(np.uint64(seed) ^ _mix64(np.uint64(frame) ^ _mix64(mols ^ _mix64(att ^ _SALT))))
        self.k = np.zeros(mols.shape, np.uint64)

    def uniform(self, sel=None):
        """Next uniform draw of the streams in ``sel`` (all by default)."""
        if sel is None:
            sel = slice(None)
        with np.errstate(over="ignore"):
            self.k[sel] += np.uint64(1)
            h = _mix64(self.base[sel] + _STEP * self.k[sel])
        return (h >> np.uint64(11)).astype(np.float64) * 2.0 ** -53

    def gauss(self):
        s = np.zeros(self.base.shape)
        for _ in range(12):
            s = s + self.uniform()
        return s - 6.0

    def _sphere(self, dim):
        out = np.zeros(self.base.shape + (dim,))
        todo = np.ones(self.base.shape, bool)
        while todo.any():
            idx = np.nonzero(todo)[0]
            c = [2.0 * self.uniform(idx) - 1.0 for _ in range(dim)]
            r2 = c[0] * c[0]
            for q in c[1:]:
                r2 = r2 + q * q
            ok = (r2 > 1e-4) & (r2 <= 1.0)
            r = np.sqrt(r2[ok])
            for d in range(dim):
                out[idx[ok], d] = c[d][ok] / r
            todo[idx[ok]] = False
        return out

    def unit3(self):
        return self._sphere(3)

    def quat(self):
        return self._sphere(4)


def cube_root(x: float) -> float:
    y = x / 3 + 0.5 if x > 1 else 1.0
    for _ in range(200):
        y = y - (y * y * y - x) / (3 * y * y)
    return y


def _trunc(f):
    return np.trunc(f)   # (double)(long long)f for |f| < 2^63


def wrap(v, L):
    f = v / L
    fl = _trunc(f)
    fl = np.where(fl > f, fl - 1.0, fl)
    return v - L * fl


def min_image(d, L):
    f = d / L
    r = _trunc(f + np.where(f >= 0, 0.5, -0.5))
    return d - L * r


def rotmat(q):
    w, x, y, z = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    R = np.empty(q.shape[:-1] + (3, 3))
    R[..., 0, 0] = 1 - 2 * (y * y + z * z)
    R[..., 0, 1] = 2 * (x * y - w * z)
    R[..., 0, 2] = 2 * (x * z + w * y)
    R[..., 1, 0] = 2 * (x * y + w * z)
    R[..., 1, 1] = 1 - 2 * (x * x + z * z)
    R[..., 1, 2] = 2 * (y * z - w * x)
    R[..., 2, 0] = 2 * (x * z - w * y)
    R[..., 2, 1] = 2 * (y * z + w * x)
    R[..., 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def qmul(a, b):
    o = np.empty(np.broadcast(a, b).shape)
    o[..., 0] = a[..., 0] * b[..., 0] - a[..., 1] * b[..., 1] - a[..., 2] * b[..., 2] - a[..., 3] * b[..., 3]
    o[..., 1] = a[..., 0] * b[..., 1] + a[..., 1] * b[..., 0] + a[..., 2] * b[..., 3] - a[..., 3] * b[..., 2]
    o[..., 2] = a[..., 0] * b[..., 2] - a[..., 1] * b[..., 3] + a[..., 2] * b[..., 0] + a[..., 3] * b[..., 1]
    o[..., 3] = a[..., 0] * b[..., 3] + a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1] + a[..., 3] * b[..., 0]
    return o


def qnorm(q):
    r = np.sqrt(q[..., 0] * q[..., 0] + q[..., 1] * q[..., 1] + q[..., 2] * q[..., 2] + q[..., 3] * q[..., 3])
    return q / r[..., None]


def sites(o, q, nsite=3):
    """Absolute positions of the first ``nsite`` sites, (..., nsite, 3), in the generator's
    order of additions."""
    R = rotmat(q)
    out = np.empty(o.shape[:-1] + (nsite, 3))
    for s in range(nsite):
        for a in range(3):
            out[..., s, a] = o[..., a] + R[..., a, 0] * BODY[s, 0] + R[..., a, 1] * BODY[s, 1] \
                + R[..., a, 2] * BODY[s, 2]
    return out


def _clash(cand, others, L, rmin2):
    """Whether each candidate's O/H sites come within sqrt(rmin2) of those of the molecule it
    is paired with: cand, others (P, 3, 3)."""
    d = min_image(cand[:, :, None, :] - others[:, None, :, :], L)
    r2 = d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1] + d[..., 2] * d[..., 2]
    return (r2 < rmin2).any(axis=(1, 2))


def _pairs_near(o_a, o_b, L, rc):
    """Index pairs (i, j) with the minimum-image O..O distance of o_a[i], o_b[j] below rc."""
    d = min_image(o_a[:, None, :] - o_b[None, :, :], L)
    r2 = (d * d).sum(-1)
    return np.nonzero(r2 < rc * rc)


def trajectory(nmol: int, nframes: int, seed: int = 1, box_nm: float = 0.0, sigma_trans: float = 0.003,
               sigma_rot_deg: float = 3.0, jitter: float = 0.02, min_contact: float = 0.15, max_tries: int = 8):
    """Positions (nframes, 4*nmol, 3) float32 and the box (3,) float32."""
    L = box_nm if box_nm > 0 else 1.2417 * cube_root(nmol / 64.0)
    rmin2 = min_contact * min_contact
    rot_sigma = sigma_rot_deg * (3.14159265358979323846 / 180.0)
    rc = min_contact + 2 * R_OH + 0.01   # an O/H contact needs an O..O distance below min_contact + 2 r_OH
    c = 1
    while c * c * c < nmol:
        c += 1
    a = L / c
    o = np.zeros((nmol, 3))
    q = np.zeros((nmol, 4))
    st_sites = np.zeros((nmol, 3, 3))
    # frame 0: molecule j checks against molecules 0..j-1 only
    for j in range(nmol):
        ix, iy, iz = j % c, (j // c) % c, j // (c * c)
        for att in range(100000):
            st = Streams(seed, 0, [j], [att])
            oj = np.empty((1, 3))
            oj[0, 0] = (ix + 0.5) * a + jitter * (2 * st.uniform()[0] - 1)
            oj[0, 1] = (iy + 0.5) * a + jitter * (2 * st.uniform()[0] - 1)
            oj[0, 2] = (iz + 0.5) * a + jitter * (2 * st.uniform()[0] - 1)
            oj = wrap(oj, L)
            qj = st.quat()
            sj = sites(oj, qj)
            bad = False
            if j > 0:
                _, near = _pairs_near(oj, o[:j], L, rc)
                if len(near):
                    bad = _clash(np.repeat(sj, len(near), 0), st_sites[near], L, rmin2).any()
            if not bad:
                o[j], q[j], st_sites[j] = oj[0], qj[0], sj[0]
                break
        else:
            raise RuntimeError(f"cannot place molecule {j} without contacts")
    out = np.empty((nframes, 4 * nmol, 3), np.float32)
    out[0] = sites(o, q, 4).reshape(-1, 3).astype(np.float32)
    mols = np.arange(nmol)
    for f in range(1, nframes):
        props = []   # props[att] = (o, q, sites) of every molecule's proposal for attempt att

        def proposal(att):
            while len(props) <= att:
                st = Streams(seed, f, mols, len(props))
                on = np.empty((nmol, 3))
                for d in range(3):
                    on[:, d] = wrap(o[:, d] + sigma_trans * st.gauss(), L)
                u = st.unit3()
                half = 0.5 * rot_sigma * st.gauss()
                dq = qnorm(np.stack([np.ones(nmol), u[:, 0] * half, u[:, 1] * half, u[:, 2] * half], 1))
                qn = qnorm(qmul(dq, q))
                props.append((on, qn, sites(on, qn)))
            return props[att]

        # every molecule is assumed to take its first proposal; `bad` marks the molecules
        # for which that fails, given the assumed states of the molecules before them.
        # They are processed in order like the generator does, and each change of a
        # molecule's state re-checks only its neighbours after it.
        p0o, p0q, p0s = proposal(0)
        new_o, new_q, new_s = p0o.copy(), p0q.copy(), p0s.copy()
        bad = _clashes_all(p0o, p0s, new_o, new_s, o, st_sites, L, rc, rmin2)
        j = -1
        while True:
            hit = np.nonzero(bad[j + 1:])[0]
            if len(hit) == 0:
                break
            j = j + 1 + int(hit[0])
            new_o[j], new_q[j], new_s[j] = o[j], q[j], st_sites[j]     # every attempt rejected
            for att in range(1, max_tries):
                po, pq, ps = proposal(att)
                if not _clash_one(j, po[j], ps[j], new_o, new_s, o, st_sites, L, rc, rmin2):
                    new_o[j], new_q[j], new_s[j] = po[j], pq[j], ps[j]
                    break
            # molecules after j near its assumed or its actual position: check them again
            near = set()
            for pos in (p0o[j], new_o[j]):
                d = min_image(p0o[j + 1:] - pos, L)
                near.update((j + 1 + np.nonzero((d * d).sum(-1) < rc * rc)[0]).tolist())
            for k in sorted(near):
                bad[k] = _clash_one(k, p0o[k], p0s[k], new_o, new_s, o, st_sites, L, rc, rmin2)
        o, q, st_sites = new_o, new_q, new_s
        out[f] = sites(o, q, 4).reshape(-1, 3).astype(np.float32)
    box = np.full(3, L, np.float32)
    return out, box


def _clashes_all(p0o, p0s, new_o, new_s, old_o, old_s, L, rc, rmin2):
    """For every molecule j: whether its first proposal touches a molecule k != j, taken in
    its new state for k < j and its old state for k > j."""
    from scipy.spatial import cKDTree
    n = len(p0o)
    bad = np.zeros(n, bool)
    def inbox(x):   # coordinates in [0, L) for the periodic tree (a prefilter only)
        y = np.mod(x, L)
        return np.where(y >= L, 0.0, y)

    tp = cKDTree(inbox(p0o), boxsize=L)
    for oth_o, oth_s, lower in ((new_o, new_s, True), (old_o, old_s, False)):
        pr = tp.sparse_distance_matrix(cKDTree(inbox(oth_o), boxsize=L), rc, output_type="ndarray")
        j, k = pr["i"].astype(np.int64), pr["j"].astype(np.int64)
        m = (k < j) if lower else (k > j)
        j, k = j[m], k[m]
        if len(j):
            cl = _clash(p0s[j], oth_s[k], L, rmin2)
            bad[j[cl]] = True
    return bad


def _clash_one(j, cand_o, cand_s, new_o, new_s, old_o, old_s, L, rc, rmin2):
    """Whether molecule j's candidate touches a molecule k != j, taken in its new state for
    k < j and its old state for k > j."""
    n = len(new_o)
    lower = (np.arange(n) < j)
    oth_o = np.where(lower[:, None], new_o, old_o)
    oth_s = np.where(lower[:, None, None], new_s, old_s)
    _, near = _pairs_near(cand_o[None], oth_o, L, rc)
    near = near[near != j]
    return bool(len(near)) and bool(_clash(np.repeat(cand_s[None], len(near), 0), oth_s[near], L, rmin2).any())
