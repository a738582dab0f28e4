"""Seeded synthetic linear systems with the reference's CSR layout.

The reference assembles its systems on a fixed CSR pattern built by
``CFVM::define_matrix_structure`` (``cfvm.cpp:74-98``): per row the diagonal,
one entry per neighbouring cell, and -- on every row whose cell touches a
boundary -- one phantom column ``(size_t)-1`` holding an exact 0, all sorted
ascending, so the phantom comes last.  Every generator here reproduces that
layout (``row_ptr``/``column_index`` as ``uint64``), so the systems can be fed
unchanged to the reference, to the oracle and to the GPU library.

Workloads (no mesh files or datasets exist for them; everything is seeded):

* ``pattern_1d``: the 1D mesh of ``generate_1d_mesh`` (cgeometry_supply.h:26-77),
  every cell a boundary cell (empty side faces).
* ``hex_pprime``: the p'-type system on an ``nx*ny*nz`` hex box over the unit
  cube with interior nodes jittered uniformly by +-10% of the spacing:
  off-diagonals ``-Gamma_f A_f / d_f`` with ``Gamma_f ~ U[0.5, 2]`` plus a
  first-order-upwind convective part from a smooth seeded velocity field scaled
  to a maximum cell Peclet number, diagonal ``ratio * sum |off|`` with
  ``ratio ~ U[1.01, 1.1]`` (the compressibility term psi V / dt), RHS
  ``U[-1, 1]``.  ``peclet=0`` gives the symmetric diffusion-only variant.
* ``tet_pprime``: the same recipe on ``nx*ny*nz`` hexes split into 6 tetrahedra
  each (Kuhn split along the (0,0,0)-(1,1,1) diagonal, conforming).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

PHANTOM = np.uint64(0xFFFFFFFFFFFFFFFF)
BASE_SEED = 20261203


@dataclass
class System:
    """One CSR system in the reference layout."""

    row_ptr: np.ndarray        # uint64[n+1]
    column_index: np.ndarray   # uint64[nnz], phantom = 2**64-1
    value: np.ndarray          # float64[nnz]
    b: np.ndarray              # float64[n]
    name: str = ""

    @property
    def n(self) -> int:
        return self.row_ptr.size - 1

    @property
    def nnz(self) -> int:
        return self.column_index.size

    @property
    def nnz_real(self) -> int:
        return int(np.count_nonzero(self.column_index != PHANTOM))


def _csr_from_slots(cols: np.ndarray, vals: np.ndarray | None, mask: np.ndarray):
    """Compress an (n, k) slot table (already in sorted column order) to CSR."""
    counts = mask.sum(axis=1)
    rp = np.zeros(cols.shape[0] + 1, np.uint64)
    np.cumsum(counts, out=rp[1:])
    col = cols[mask].astype(np.uint64)
    val = vals[mask] if vals is not None else None
    return rp, col, val


def pattern_1d(ncells: int):
    """CSR pattern of the reference's 1D mesh: rows [i-1, i, i+1, phantom]."""
    i = np.arange(ncells, dtype=np.int64)
    cols = np.stack([i - 1, i, i + 1, np.full_like(i, -1)], axis=1)
    mask = np.stack([i > 0, np.ones_like(i, bool), i < ncells - 1, np.ones_like(i, bool)], axis=1)
    cols_u = cols.astype(np.uint64)  # -1 -> 2**64-1, the reference's phantom
    rp, col, _ = _csr_from_slots(cols_u, None, mask)
    return rp, col


def hex_pattern(nx: int, ny: int, nz: int):
    """7-point pattern in natural order (cell = i + nx*(j + ny*k)) with phantoms."""
    rp, col, _, _ = _hex_slots(nx, ny, nz)
    return rp, col


def _hex_slots(nx, ny, nz):
    n = nx * ny * nz
    c = np.arange(n, dtype=np.int64)
    i = c % nx
    j = (c // nx) % ny
    k = c // (nx * ny)
    nxy = nx * ny
    cols = np.stack([c - nxy, c - nx, c - 1, c, c + 1, c + nx, c + nxy,
                     np.full_like(c, -1)], axis=1)
    boundary = (i == 0) | (i == nx - 1) | (j == 0) | (j == ny - 1) | (k == 0) | (k == nz - 1)
    mask = np.stack([k > 0, j > 0, i > 0, np.ones(n, bool), i < nx - 1, j < ny - 1,
                     k < nz - 1, boundary], axis=1)
    rp, col, _ = _csr_from_slots(cols.astype(np.uint64), None, mask)
    return rp, col, cols, mask


def _jittered_nodes(nx, ny, nz, rng, jitter=0.1):
    hx, hy, hz = 1.0 / nx, 1.0 / ny, 1.0 / nz
    X, Y, Z = np.meshgrid(np.arange(nx + 1) * hx, np.arange(ny + 1) * hy,
                          np.arange(nz + 1) * hz, indexing="ij")
    P = np.stack([X, Y, Z], axis=-1)  # (nx+1, ny+1, nz+1, 3)
    J = rng.uniform(-jitter, jitter, size=P.shape) * np.array([hx, hy, hz])
    interior = np.zeros(P.shape[:3], bool)
    interior[1:-1, 1:-1, 1:-1] = True
    P[interior] += J[interior]
    return P


def _velocity(points, rng):
    """Smooth seeded field: a sum of three sinusoidal modes per component."""
    u = np.zeros_like(points)
    for _ in range(3):
        kvec = rng.uniform(1.0, 4.0, size=3) * np.pi
        phase = rng.uniform(0, 2 * np.pi, size=3)
        amp = rng.uniform(-1.0, 1.0, size=3)
        arg = points @ kvec
        for d in range(3):
            u[..., d] += amp[d] * np.sin(arg + phase[d])
    return u


def _assemble(n, L, R, D, F, ratio, slot_L, slot_R, cols, mask):
    """Fill an (n, k) slot table from face coefficients; returns CSR values.

    Face f joins cells L < R.  Upwind convection with face flux F (positive
    from L to R):  a_LR = -D - max(-F, 0),  a_RL = -D - max(F, 0).
    """
    vals = np.zeros(cols.shape, np.float64)
    aLR = -D - np.maximum(-F, 0.0)
    aRL = -D - np.maximum(F, 0.0)
    vals[L, slot_L] = aLR          # row L, column R
    vals[R, slot_R] = aRL          # row R, column L
    offsum = np.zeros(n)
    np.add.at(offsum, L, np.abs(aLR))
    np.add.at(offsum, R, np.abs(aRL))
    diag_slot = np.argmax(cols == np.arange(n)[:, None], axis=1)
    vals[np.arange(n), diag_slot] = ratio * offsum
    return vals[mask]


def hex_pprime(nx: int, ny: int | None = None, nz: int | None = None, *, peclet: float = 10.0,
               seed: int = BASE_SEED, jitter: float = 0.1) -> System:
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    n = nx * ny * nz
    rp, col, cols, mask = _hex_slots(nx, ny, nz)
    P = _jittered_nodes(nx, ny, nz, np.random.default_rng(seed), jitter)
    cent = 0.125 * sum(P[a:a + nx, b:b + ny, c:c + nz] for a in (0, 1) for b in (0, 1)
                       for c in (0, 1))
    cent = cent.transpose(2, 1, 0, 3).reshape(n, 3)  # cell = i + nx*(j + ny*k)

    Ls, Rs, Av, Fc, SL, SR = [], [], [], [], [], []
    idx = np.arange(n).reshape(nz, ny, nx)
    # x-faces: between (i,j,k) and (i+1,j,k); face nodes at x-index i+1
    for axis, (sl, sr) in enumerate(((4, 2), (5, 1), (6, 0))):
        if axis == 0:
            Lc, Rc = idx[:, :, :-1].ravel(), idx[:, :, 1:].ravel()
            q = P[1:nx, :, :]
            n00, n10, n01, n11 = q[:, :-1, :-1], q[:, 1:, :-1], q[:, :-1, 1:], q[:, 1:, 1:]
            order = (2, 1, 0)
        elif axis == 1:
            Lc, Rc = idx[:, :-1, :].ravel(), idx[:, 1:, :].ravel()
            q = P[:, 1:ny, :]
            n00, n10, n01, n11 = q[:-1, :, :-1], q[:-1, :, 1:], q[1:, :, :-1], q[1:, :, 1:]
            order = (2, 1, 0)
        else:
            Lc, Rc = idx[:-1, :, :].ravel(), idx[1:, :, :].ravel()
            q = P[:, :, 1:nz]
            n00, n10, n01, n11 = q[:-1, :-1, :], q[1:, :-1, :], q[:-1, 1:, :], q[1:, 1:, :]
            order = (2, 1, 0)
        area = 0.5 * np.cross(n11 - n00, n01 - n10)
        fc = 0.25 * (n00 + n10 + n01 + n11)
        area = area.transpose(*order, 3).reshape(-1, 3)
        fc = fc.transpose(*order, 3).reshape(-1, 3)
        Ls.append(Lc); Rs.append(Rc); Av.append(area); Fc.append(fc)
        SL.append(np.full(Lc.size, sl)); SR.append(np.full(Lc.size, sr))
    L = np.concatenate(Ls); R = np.concatenate(Rs); A = np.concatenate(Av)
    FC = np.concatenate(Fc); slot_L = np.concatenate(SL); slot_R = np.concatenate(SR)
    dvec = cent[R] - cent[L]
    # orient the area vector from L to R
    sgn = np.sign(np.einsum("ij,ij->i", A, dvec))
    A *= sgn[:, None]
    Amag = np.linalg.norm(A, axis=1)
    dist = np.linalg.norm(dvec, axis=1)
    rng1 = np.random.default_rng(seed + 1)
    gamma = rng1.uniform(0.5, 2.0, size=L.size)
    D = gamma * Amag / dist
    F = np.zeros(L.size)
    if peclet > 0:
        u = _velocity(FC, np.random.default_rng(seed + 2))
        F = np.einsum("ij,ij->i", u, A)
        F *= peclet / np.max(np.abs(F) / D)
    ratio = np.random.default_rng(seed + 3).uniform(1.01, 1.1, size=n)
    val = _assemble(n, L, R, D, F, ratio, slot_L, slot_R, cols, mask)
    b = np.random.default_rng(seed + 4).uniform(-1.0, 1.0, size=n)
    name = f"hex{nx}x{ny}x{nz}_pe{peclet:g}"
    return System(rp, col, val, b, name)


# Kuhn split of a unit cube into 6 tetrahedra along the (0,0,0)-(1,1,1) diagonal:
# one tet per axis permutation.  Local corner id = dx + 2*dy + 4*dz.
def _kuhn_tets():
    import itertools
    tets = []
    for perm in itertools.permutations(range(3)):
        v = [0, 0, 0]
        corners = [0]
        for ax in perm:
            v[ax] = 1
            corners.append(v[0] + 2 * v[1] + 4 * v[2])
        tets.append(corners)
    return np.array(tets, np.int64)  # (6, 4)


def _tet_mesh(nx, ny, nz, seed, jitter):
    """Kuhn-split tet mesh of the jittered box: node coordinates, cell
    vertices, centroids, the interior faces (L < R, sorted by vertex key) with
    their area vectors (oriented L -> R) and centres, and the boundary faces
    (cell, vertex triple)."""
    nh = nx * ny * nz
    n = 6 * nh
    P = _jittered_nodes(nx, ny, nz, np.random.default_rng(seed), jitter)
    node_id = np.arange((nx + 1) * (ny + 1) * (nz + 1)).reshape(nx + 1, ny + 1, nz + 1)
    h = np.arange(nh)
    hi, hj, hk = h % nx, (h // nx) % ny, h // (nx * ny)
    corner = np.empty((nh, 8), np.int64)
    for cid in range(8):
        dx, dy, dz = cid & 1, (cid >> 1) & 1, (cid >> 2) & 1
        corner[:, cid] = node_id[hi + dx, hj + dy, hk + dz]
    kt = _kuhn_tets()
    tv = corner[:, kt].reshape(n, 4)            # cell = 6*hex + local tet
    X = P.reshape(-1, 3)
    cent = X[tv].mean(axis=1)
    faces = np.stack([np.sort(np.delete(tv, m, axis=1), axis=1) for m in range(4)], axis=1)
    fkeys = faces.reshape(-1, 3)
    owner = np.repeat(np.arange(n), 4)
    order = np.lexsort((fkeys[:, 2], fkeys[:, 1], fkeys[:, 0]))
    fs = fkeys[order]
    same = np.all(fs[1:] == fs[:-1], axis=1)
    a_idx = order[:-1][same]
    b_idx = order[1:][same]
    ca, cb = owner[a_idx], owner[b_idx]
    L = np.minimum(ca, cb)
    R = np.maximum(ca, cb)
    fnodes = fkeys[a_idx]
    p0, p1, p2 = X[fnodes[:, 0]], X[fnodes[:, 1]], X[fnodes[:, 2]]
    A = 0.5 * np.cross(p1 - p0, p2 - p0)
    FC = (p0 + p1 + p2) / 3.0
    dvec = cent[R] - cent[L]
    A *= np.sign(np.einsum("ij,ij->i", A, dvec))[:, None]
    paired = np.zeros(fkeys.shape[0], bool)
    paired[a_idx] = True
    paired[b_idx] = True
    bidx = np.nonzero(~paired)[0]
    return n, X, tv, cent, L, R, A, FC, dvec, owner[bidx], fkeys[bidx]


def tet_pprime(nx: int, ny: int | None = None, nz: int | None = None, *, peclet: float = 50.0,
               seed: int = BASE_SEED, jitter: float = 0.1) -> System:
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    n, X, tv, cent, L, R, A, FC, dvec, _, _ = _tet_mesh(nx, ny, nz, seed, jitter)
    Amag = np.linalg.norm(A, axis=1)
    dist = np.linalg.norm(dvec, axis=1)
    # boundary cells: tets with fewer than 4 interior faces
    nint = np.bincount(np.concatenate([L, R]), minlength=n)
    boundary = nint < 4
    # CSR slots: diag + neighbours sorted, phantom last
    deg = nint + 1
    rows = np.concatenate([np.arange(n), L, R])
    cols_ = np.concatenate([np.arange(n), R, L])
    ordr = np.lexsort((cols_, rows))
    rows, cols_ = rows[ordr], cols_[ordr]
    rp_real = np.zeros(n + 1, np.int64)
    np.cumsum(deg, out=rp_real[1:])
    # insert phantoms
    counts = deg + boundary.astype(np.int64)
    rp = np.zeros(n + 1, np.uint64)
    np.cumsum(counts, out=rp[1:])
    col = np.empty(int(rp[-1]), np.uint64)
    pos_real = np.arange(rows.size) - rp_real[rows] + rp[rows].astype(np.int64)
    col[pos_real] = cols_.astype(np.uint64)
    col[(rp[1:].astype(np.int64) - 1)[boundary]] = PHANTOM
    # values
    rng1 = np.random.default_rng(seed + 1)
    gamma = rng1.uniform(0.5, 2.0, size=L.size)
    D = gamma * Amag / dist
    F = np.zeros(L.size)
    if peclet > 0:
        u = _velocity(FC, np.random.default_rng(seed + 2))
        F = np.einsum("ij,ij->i", u, A)
        F *= peclet / np.max(np.abs(F) / D)
    aLR = -D - np.maximum(-F, 0.0)
    aRL = -D - np.maximum(F, 0.0)
    val = np.zeros(col.size)
    # position of (L, R) in row L and (R, L) in row R via searchsorted on keys
    key_pos = pos_real
    key = rows * np.int64(n) + cols_
    def where(r, c):
        return key_pos[np.searchsorted(key, r * np.int64(n) + c)]
    val[where(L, R)] = aLR
    val[where(R, L)] = aRL
    offsum = np.zeros(n)
    np.add.at(offsum, L, np.abs(aLR))
    np.add.at(offsum, R, np.abs(aRL))
    ratio = np.random.default_rng(seed + 3).uniform(1.01, 1.1, size=n)
    val[where(np.arange(n), np.arange(n))] = ratio * offsum
    b = np.random.default_rng(seed + 4).uniform(-1.0, 1.0, size=n)
    return System(rp, col, val, b, f"tet{nx}x{ny}x{nz}_pe{peclet:g}")


def random_rows_system(n: int, max_row: int, seed: int = 7, phantom_frac: float = 0.3) -> System:
    """Ragged, diagonally dominant system with random sorted row patterns
    (1..max_row entries per row, diagonal always present, some phantoms)."""
    rng = np.random.default_rng(seed)
    rows = []
    for i in range(n):
        k = int(rng.integers(0, max_row))
        nb = rng.choice(n, size=min(k, n), replace=False) if n > 1 else np.array([], int)
        cs = sorted(set(int(c) for c in nb) | {i})
        rows.append(cs)
    rp = np.zeros(n + 1, np.uint64)
    cols, vals = [], []
    for i, cs in enumerate(rows):
        rowv = list(rng.uniform(-1.0, 1.0, size=len(cs)))
        s = sum(abs(v) for c, v in zip(cs, rowv) if c != i)
        rowv = [(s * rng.uniform(1.05, 1.5) + 0.1) if c == i else v for c, v in zip(cs, rowv)]
        cols.extend(cs)
        vals.extend(rowv)
        if rng.uniform() < phantom_frac:
            cols.append(int(PHANTOM))
            vals.append(0.0)
        rp[i + 1] = len(cols)
    return System(rp, np.array(cols, np.uint64), np.array(vals), rng.uniform(-1, 1, size=n),
                  f"random{n}_r{max_row}")


@dataclass
class FlowCase:
    """A finite-volume mesh with a flow state in the argument form of the
    face-loop assembly (ocsl_set_faces / ocsl_assemble_device): the
    reference-layout pattern, face connectivity, the per-field state arrays
    and the equation settings."""
    name: str
    row_ptr: np.ndarray
    column_index: np.ndarray
    left: np.ndarray
    right: np.ndarray
    bc_left: np.ndarray
    state: dict
    eq: dict
    inlet: np.ndarray  # boundary faces on x = 0 (the inlet set)

    @property
    def n(self) -> int:
        return self.row_ptr.size - 1


AIR = {"R_specific": 8.31446261815324 / (28.9651159 / 1000.0), "gamma": 1.4,
       "sutherland": (1.458e-6, 110.4), "prandtl": 0.713}


def hex_flow_state(nx: int, ny: int | None = None, nz: int | None = None, *, seed: int = 20261203,
                   equation: int = 1, transient: bool = True, blended: bool = True,
                   inlet_value: float = 0.0) -> FlowCase:
    """Seeded flow state on an nx*ny*nz unit-box hex mesh for the assembly.

    Interior faces in x-, then y-, then z-direction order; boundary faces:
    x = 0 a supersonic inlet (its pressure-correction term is the Dirichlet
    term a_PP += D, b_P += D * p_in of solvers_common.h:56-67 with
    p_in = ``inlet_value``), x = 1 a subsonic pressure outlet, the other four
    sides slip walls.  Fields: T = 300 K +- 20 K and a smooth seeded velocity
    (3 sinusoidal modes, ~100 m/s); density from the ideal gas at p = 1e5 Pa;
    face mass flow rho_f (u_f . A); Qy ~ U[0.5, 2] x scale (seed + 1), so the
    pressure-correction system is diffusion-dominated with a convective part
    (cell Peclet ~ 0.4 at 128^3) and a transient diagonal (dt = 1e-4 s)."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    rp, col = hex_pattern(nx, ny, nz)
    h = np.array([1.0 / nx, 1.0 / ny, 1.0 / nz])
    c = np.arange(n, dtype=np.int64)
    ijk = np.stack([c % nx, (c // nx) % ny, c // (nx * ny)], axis=1)
    centers = (ijk + 0.5) * h
    vel = 100.0 * (1.0 + 0.2 * _velocity(centers, rng))  # (n, 3), mostly +x
    T = 300.0 + 20.0 * np.sin(2 * np.pi * centers[:, 0]) * np.cos(np.pi * centers[:, 1])
    p = np.full(n, 1.0e5)
    rho = p / AIR["R_specific"] / T
    strides = (1, nx, nx * ny)
    dims = (nx, ny, nz)
    left, right, axis = [], [], []
    for a in range(3):
        m = ijk[:, a] < dims[a] - 1
        left.append(c[m])
        right.append(c[m] + strides[a])
        axis.append(np.full(int(m.sum()), a))
    left, right, axis = np.concatenate(left), np.concatenate(right), np.concatenate(axis)
    area = np.where(axis == 0, h[1] * h[2], np.where(axis == 1, h[0] * h[2], h[0] * h[1]))
    dist = h[axis]
    rho_f = 0.5 * (rho[left] + rho[right])
    un = 0.5 * (vel[left, axis] + vel[right, axis])
    mdot = rho_f * un * area
    # Qy sized so that the six faces' D = Qy rho_f sum to ~20x the transient
    # diagonal vol / (dt R T gamma): diagonal dominance ~1.05, as a p' system
    dt = 1e-4
    qy_scale = 20.0 / 6.0 * h.prod() / (dt * AIR["R_specific"] * 300.0 * AIR["gamma"] * rho_f)
    qy = np.random.default_rng(seed + 1).uniform(0.5, 2.0, left.size) * qy_scale
    # boundary faces: (cell, outward axis, sign)
    bl, bt, ba, bs = [], [], [], []
    for a in range(3):
        for side, sign in ((0, -1.0), (dims[a] - 1, 1.0)):
            cells = c[ijk[:, a] == side]
            bl.append(cells)
            ba.append(np.full(cells.size, a))
            bs.append(np.full(cells.size, sign))
            if a == 0:
                kind = _abi_bc("SUPERSONIC_INLET") if sign < 0 else _abi_bc("PRESSURE_OUTLET")
            else:
                kind = _abi_bc("WALL")
            bt.append(np.full(cells.size, kind))
    bc_left, bc_type = np.concatenate(bl), np.concatenate(bt).astype(np.int32)
    bc_axis, bc_sign = np.concatenate(ba), np.concatenate(bs)
    nb = bc_left.size
    bc_area = np.where(bc_axis == 0, h[1] * h[2], np.where(bc_axis == 1, h[0] * h[2], h[0] * h[1]))
    bc_av = np.zeros((3, nb))
    bc_av[bc_axis, np.arange(nb)] = bc_sign * bc_area
    bc_vel = vel[bc_left].T.copy()
    bc_rho = rho[bc_left]
    bc_mdot = bc_rho * (bc_vel[bc_axis, np.arange(nb)] * bc_sign) * bc_area
    bc_mdot[bc_type == _abi_bc("WALL")] = 0.0
    inlet = np.nonzero(bc_type == _abi_bc("SUPERSONIC_INLET"))[0]
    bc_value = np.zeros(nb)
    bc_value[inlet] = inlet_value
    vol = np.full(n, h[0] * h[1] * h[2])
    state = {
        "geo_aver": np.full(left.size, 0.5), "ksi_A": area / dist, "mdot": mdot,
        "density": rho_f, "qy": qy, "stress": np.zeros((3, left.size)),
        "bc_type": bc_type, "bc_wall": np.full(nb, 1, np.int32),
        "bc_supersonic": np.zeros(nb, np.int32), "bc_area": bc_area, "bc_area_vector": bc_av,
        "bc_perp_dist": 0.5 * h[bc_axis], "bc_ksi_A": bc_area / (0.5 * h[bc_axis]),
        "bc_mdot": bc_mdot, "bc_density": bc_rho, "bc_qy": np.full(nb, float(np.mean(qy))),
        "bc_temperature": T[bc_left], "bc_enthalpy": 1005.0 * T[bc_left],
        "bc_velocity": bc_vel, "bc_value": bc_value,
        "volume": vol, "delta_t": np.full(n, dt), "velocity": vel.T.copy(),
        "velocity_last": vel.T.copy(), "pressure_grad": np.zeros((3, n)), "density_c": rho,
        "density_last": rho * (1.0 + 1e-4 * np.sin(7.0 * centers[:, 2])), "pressure": p,
        "pressure_last": p.copy(), "pressure_corr": np.zeros(n), "temperature": T,
        "enthalpy": 1005.0 * T, "enthalpy_last": 1005.0 * T,
    }
    eq = dict(AIR, equation=equation, dimension=0, viscous=0, blended=int(blended),
              transient=int(transient), implicit_underrelaxation=0.7)
    return FlowCase(f"hexflow{nx}x{ny}x{nz}", rp, col, left.astype(np.int32),
                    right.astype(np.int32), bc_left.astype(np.int32), state, eq, inlet)


def tet_flow_state(nx: int, ny: int | None = None, nz: int | None = None, *,
                   seed: int = BASE_SEED + 7, jitter: float = 0.1, equation: int = 1,
                   transient: bool = True, blended: bool = True,
                   inlet_value: float = 0.0) -> FlowCase:
    """Seeded flow state on the Kuhn-split tet mesh of a jittered nx*ny*nz box
    (6 tets per hex), in the same form as hex_flow_state but with general
    geometry: interior faces in vertex-key order, geo_aver from the face-centre
    distances (cfvm.cpp:137), ksi_A = |A| / d, tet volumes; boundary faces on
    x = 0 a supersonic inlet, x = 1 a pressure outlet, walls elsewhere, with
    outward area vectors and the centroid's distance to the face plane."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    n, X, tv, cent, L, R, A, FC, dvec, bcell, bnodes = _tet_mesh(nx, ny, nz, seed, jitter)
    rng = np.random.default_rng(seed + 11)
    Amag = np.linalg.norm(A, axis=1)
    dist = np.linalg.norm(dvec, axis=1)
    dL = np.linalg.norm(FC - cent[L], axis=1)
    dR = np.linalg.norm(cent[R] - FC, axis=1)
    geo = dR / (dL + dR)
    vel = 100.0 * (1.0 + 0.2 * _velocity(cent, rng))
    T = 300.0 + 20.0 * np.sin(2 * np.pi * cent[:, 0]) * np.cos(np.pi * cent[:, 1])
    p = np.full(n, 1.0e5)
    rho = p / AIR["R_specific"] / T
    rho_f = geo * rho[L] + (1.0 - geo) * rho[R]
    u_f = geo[:, None] * vel[L] + (1.0 - geo[:, None]) * vel[R]
    mdot = rho_f * np.einsum("ij,ij->i", u_f, A)
    e1, e2, e3 = (X[tv[:, k]] - X[tv[:, 0]] for k in (1, 2, 3))
    vol = np.abs(np.einsum("ij,ij->i", e1, np.cross(e2, e3))) / 6.0
    dt = 1e-4
    qy = np.random.default_rng(seed + 1).uniform(0.5, 2.0, L.size) * (
        20.0 / 4.0 * vol.mean() / (dt * AIR["R_specific"] * 300.0 * AIR["gamma"] * rho_f))
    # boundary faces: outward area vector, plane distance, kind by position
    q0, q1, q2 = X[bnodes[:, 0]], X[bnodes[:, 1]], X[bnodes[:, 2]]
    bav = 0.5 * np.cross(q1 - q0, q2 - q0)
    bfc = (q0 + q1 + q2) / 3.0
    out = np.einsum("ij,ij->i", bav, bfc - cent[bcell])
    bav *= np.sign(out)[:, None]
    bc_area = np.linalg.norm(bav, axis=1)
    perp = np.abs(np.einsum("ij,ij->i", bav, bfc - cent[bcell])) / bc_area
    nb = bcell.size
    bc_type = np.full(nb, _abi_bc("WALL"), np.int32)
    bc_type[bfc[:, 0] < 1e-12] = _abi_bc("SUPERSONIC_INLET")
    bc_type[bfc[:, 0] > 1.0 - 1e-12] = _abi_bc("PRESSURE_OUTLET")
    bc_vel = vel[bcell].T.copy()
    bc_rho = rho[bcell]
    bc_mdot = bc_rho * np.einsum("ij,ij->i", vel[bcell], bav)
    bc_mdot[bc_type == _abi_bc("WALL")] = 0.0
    inlet = np.nonzero(bc_type == _abi_bc("SUPERSONIC_INLET"))[0]
    bc_value = np.zeros(nb)
    bc_value[inlet] = inlet_value
    # the reference's pattern for this face connectivity (host-only builder)
    from . import build_pattern

    rp, col = build_pattern(n, L.astype(np.int32), R.astype(np.int32), bcell.astype(np.int32))
    stress = np.random.default_rng(seed + 3).uniform(-1.0, 1.0, (3, L.size)) * 1e-3
    state = {
        "geo_aver": geo, "ksi_A": Amag / dist, "mdot": mdot, "density": rho_f, "qy": qy,
        "stress": stress, "bc_type": bc_type, "bc_wall": np.full(nb, 1, np.int32),
        "bc_supersonic": np.zeros(nb, np.int32), "bc_area": bc_area, "bc_area_vector": bav.T.copy(),
        "bc_perp_dist": perp, "bc_ksi_A": bc_area / perp, "bc_mdot": bc_mdot,
        "bc_density": bc_rho, "bc_qy": np.full(nb, float(np.mean(qy))),
        "bc_temperature": T[bcell], "bc_enthalpy": 1005.0 * T[bcell], "bc_velocity": bc_vel,
        "bc_value": bc_value, "bc_thermal": (np.arange(nb) % 2).astype(np.int32),
        "volume": vol, "delta_t": np.full(n, dt), "velocity": vel.T.copy(),
        "velocity_last": (0.99 * vel).T.copy(),
        "pressure_grad": np.random.default_rng(seed + 4).uniform(-1.0, 1.0, (3, n)),
        "density_c": rho, "density_last": rho * (1.0 + 1e-4 * np.sin(7.0 * cent[:, 2])),
        "pressure": p, "pressure_last": p.copy(),
        "pressure_corr": np.random.default_rng(seed + 5).uniform(-1.0, 1.0, n),
        "temperature": T, "enthalpy": 1005.0 * T, "enthalpy_last": 1005.0 * T * 0.999,
    }
    eq = dict(AIR, equation=equation, dimension=0, viscous=0, blended=int(blended),
              transient=int(transient), implicit_underrelaxation=0.7)
    return FlowCase(f"tetflow{nx}x{ny}x{nz}", rp, col, L.astype(np.int32), R.astype(np.int32),
                    bcell.astype(np.int32), state, eq, inlet)


def _abi_bc(name: str) -> int:
    from . import _abi

    return getattr(_abi, "BC_" + name)


@dataclass
class BatchSystem:
    system: System       # matrix (reference layout) and its first right-hand side
    rhs: np.ndarray      # [nrhs][n] right-hand sides sharing the matrix
    kind: str            # "pprime" or "momentum"


def batch_boxes(count: int = 64, *, seed: int = BASE_SEED + 40, min_cells: int = 10_000,
                max_cells: int = 500_000) -> list[tuple[int, int, int]]:
    """Box dimensions of the batching workload: cell counts log-uniform in
    [min_cells, max_cells], aspect ratios U[1, 4] per axis (seeded)."""
    rng = np.random.default_rng(seed)
    dims = []
    for _ in range(count):
        cells = float(np.exp(rng.uniform(np.log(min_cells), np.log(max_cells))))
        aspect = rng.uniform(1.0, 4.0, size=3)
        base = (cells / aspect.prod()) ** (1.0 / 3.0)
        d = np.maximum(2, np.rint(base * aspect)).astype(int)
        dims.append((int(d[0]), int(d[1]), int(d[2])))
    return dims


def batch_systems(count: int = 64, *, seed: int = BASE_SEED + 40, min_cells: int = 10_000,
                  max_cells: int = 500_000) -> list[BatchSystem]:
    """The batching workload: for each box one pressure-correction system
    (the hex p' recipe, Peclet <= 10, one right-hand side) and one momentum
    system (the same recipe at Peclet <= 50 with a stronger transient
    diagonal, three right-hand sides sharing the matrix)."""
    out = []
    for k, (nx, ny, nz) in enumerate(batch_boxes(count, seed=seed, min_cells=min_cells,
                                                 max_cells=max_cells)):
        s = hex_pprime(nx, ny, nz, peclet=10.0, seed=seed + 100 * k)
        out.append(BatchSystem(s, s.b[None, :].copy(), "pprime"))
        m = hex_pprime(nx, ny, nz, peclet=50.0, seed=seed + 100 * k + 50)
        rhs = np.random.default_rng(seed + 100 * k + 60).uniform(-1.0, 1.0, size=(3, m.n))
        out.append(BatchSystem(m, rhs, "momentum"))
    return out


def write_su2_box(path: str, nx: int, ny: int, nz: int, *, lengths=(1.0, 0.2, 0.1),
                  jitter: float = 0.1, seed: int = BASE_SEED + 70, cells: str = "hex") -> dict:
    """Write a seeded nx*ny*nz box mesh in SU2 ASCII (the format the reference
    reads, cgeometry_supply.h:201-433): interior nodes jittered by +-jitter
    of the spacing; hexahedra (type 12), each hex split into 6 Kuhn tetrahedra
    (type 10), or each hex split into 2 wedges (type 13) along its (x, y)
    diagonal; three markers in this order -- "inlet" (x = 0), "walls" (the four
    sides), "outlet" (x = lengths[0]) -- as quads (type 9) and, where the
    cells split a box face, triangles (type 5).  Returns the counts."""
    rng = np.random.default_rng(seed)
    P = _jittered_nodes(nx, ny, nz, rng, jitter) * np.asarray(lengths, float)
    nid = np.arange((nx + 1) * (ny + 1) * (nz + 1)).reshape(nx + 1, ny + 1, nz + 1)
    X = P.reshape(-1, 3)
    h = np.arange(nx * ny * nz)
    hi, hj, hk = h % nx, (h // nx) % ny, h // (nx * ny)
    corner = np.empty((h.size, 8), np.int64)  # lexicographic corners: bit 0 x, 1 y, 2 z
    for cid in range(8):
        corner[:, cid] = nid[hi + (cid & 1), hj + ((cid >> 1) & 1), hk + ((cid >> 2) & 1)]
    if cells == "hex":
        vtk = corner[:, [0, 1, 3, 2, 4, 5, 7, 6]]  # SU2 / VTK hexahedron order
        elems = [(12, row) for row in vtk]
    elif cells == "tet":
        tets = corner[:, _kuhn_tets()].reshape(-1, 4)
        # positive orientation ((p1 - p0) . ((p2 - p0) x (p3 - p0)) > 0), the one
        # whose faces' normals the reader computes pointing out of the cell
        p0, p1, p2, p3 = (X[tets[:, k]] for k in range(4))
        neg = np.einsum("ij,ij->i", p1 - p0, np.cross(p2 - p0, p3 - p0)) < 0
        tets[neg] = tets[neg][:, [0, 1, 3, 2]]
        elems = [(10, row) for row in tets]
    elif cells == "wedge":  # prisms (c0, c1, c3 | c4, c5, c7) and (c0, c3, c2 | c4, c7, c6)
        elems = []
        for row in corner:
            elems.append((13, row[[0, 1, 3, 4, 5, 7]]))
            elems.append((13, row[[0, 3, 2, 4, 7, 6]]))
    else:
        raise ValueError(cells)

    def quads(fixed_axis, value):
        out = []
        dims = [nx, ny, nz]
        a, b = [ax for ax in range(3) if ax != fixed_axis]
        for u in range(dims[a]):
            for v in range(dims[b]):
                idx = [0, 0, 0]
                idx[fixed_axis] = value
                c = []
                for du, dv in ((0, 0), (1, 0), (1, 1), (0, 1)):
                    idx[a], idx[b] = u + du, v + dv
                    c.append(nid[tuple(idx)])
                out.append((c, fixed_axis))
        return out

    markers = {"inlet": quads(0, 0),
               "walls": quads(1, 0) + quads(1, ny) + quads(2, 0) + quads(2, nz),
               "outlet": quads(0, nx)}
    with open(path, "w") as f:
        f.write("NDIME= 3\n")
        f.write(f"NELEM= {len(elems)}\n")
        for k, (t, row) in enumerate(elems):
            f.write(f"{t} " + " ".join(str(int(v)) for v in row) + f" {k}\n")
        f.write(f"NPOIN= {X.shape[0]}\n")
        for k, p in enumerate(X):
            f.write(f"{p[0]:.17g} {p[1]:.17g} {p[2]:.17g} {k}\n")
        f.write(f"NMARK= {len(markers)}\n")
        for name, faces in markers.items():
            f.write(f"MARKER_TAG= {name}\n")
            # a split cell face is two triangles along the diagonal from its lowest
            # to its highest corner (the Kuhn split; the wedges' z faces)
            elements = []
            for q, axis in faces:
                a, b, c, d = q
                split = cells == "tet" or (cells == "wedge" and axis == 2)
                if split:
                    elements += [(5, (a, b, c)), (5, (a, c, d))]
                else:
                    elements.append((9, q))
            f.write(f"MARKER_ELEMS= {len(elements)}\n")
            for t, nodes in elements:
                f.write(f"{t} " + " ".join(str(int(v)) for v in nodes) + "\n")
    return {"cells": len(elems), "nodes": X.shape[0]}
