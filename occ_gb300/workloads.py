"""Seeded synthetic inputs with the shapes of the benchmark configurations.

water()                 O at the origin, H at (+-0.757, 0.586, 0) Angstrom
water_cluster(n, box)   n rigid waters, centres uniform in a cube of side
                        `box` Angstrom, O-O >= 2.6 Angstrom by rejection,
                        uniformly random orientations (unit quaternions)
alkane(n)               n-CnH(2n+2), all-anti, C-C 1.54, C-H 1.09 Angstrom,
                        tetrahedral angles
random_density(nbf, k)  mo.D = C_occ C_occ^T with C_occ the first k columns
                        of a seeded random orthonormal nbf x nbf matrix
perturbed(D, norm, s)   D plus seeded symmetric noise of Frobenius norm `norm`
                        (a stand-in for the density change of one SCF iteration)
"""
import numpy as np

from .xc import AOBasis, Molecule

WATER_Z = [8, 1, 1]
WATER_XYZ = np.array([[0.0, 0.0, 0.0], [0.757, 0.586, 0.0], [-0.757, 0.586, 0.0]])


def water():
    return Molecule(WATER_Z, WATER_XYZ)


def _random_rotation(rng):
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([
        [a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
        [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
        [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d],
    ])


def water_cluster(n, box=10.0, seed=0, min_oo=2.6, max_tries=200000):
    rng = np.random.default_rng(seed)
    centres = []
    tries = 0
    while len(centres) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError(f"cannot place {n} waters in a {box} Angstrom box")
        c = rng.uniform(0.0, box, 3)
        if all(np.linalg.norm(c - o) >= min_oo for o in centres):
            centres.append(c)
    Z, xyz = [], []
    for c in centres:
        R = _random_rotation(rng)
        for z, r in zip(WATER_Z, WATER_XYZ):
            Z.append(z)
            xyz.append(c + R @ r)
    return Molecule(Z, np.array(xyz))


def alkane(n):
    """All-anti n-alkane CnH(2n+2): carbon zig-zag in the xy plane, two H per
    carbon above and below that plane, one more H on each terminal carbon
    where the zig-zag would continue; every angle tetrahedral."""
    if n < 2:
        raise ValueError("alkane needs at least two carbons")
    cc, ch = 1.54, 1.09
    half = np.arccos(-1.0 / 3.0) / 2.0  # half the tetrahedral angle

    def site(i):
        return np.array([i * cc * np.sin(half), (i % 2) * cc * np.cos(half), 0.0])

    carbons = [site(i) for i in range(n)]
    Z = [6] * n
    xyz = list(carbons)
    zhat = np.array([0.0, 0.0, 1.0])
    for i, c in enumerate(carbons):
        a = site(i - 1) - c
        b = site(i + 1) - c
        a /= np.linalg.norm(a)
        b /= np.linalg.norm(b)
        u = -(a + b)
        u /= np.linalg.norm(u)
        for s in (1.0, -1.0):
            Z.append(1)
            xyz.append(c + ch * (np.cos(half) * u + s * np.sin(half) * zhat))
        if i == 0:
            Z.append(1)
            xyz.append(c + ch * a)
        if i == n - 1:
            Z.append(1)
            xyz.append(c + ch * b)
    return Molecule(Z, np.array(xyz))


def random_density(nbf, nocc, seed=0):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((nbf, nbf)))
    C = Q[:, :nocc]
    return C @ C.T


def random_density_unrestricted(nbf, nalpha, nbeta, seed=0):
    """OCC's unrestricted mo.D (2 nbf x nbf, alpha block above beta, each
    0.5 C_s C_s^T, src/qm/orb.h:68-83) from seeded orthonormal orbitals,
    different for the two spins."""
    rng = np.random.default_rng(seed)
    Qa, _ = np.linalg.qr(rng.standard_normal((nbf, nbf)))
    Qb, _ = np.linalg.qr(rng.standard_normal((nbf, nbf)))
    Ca, Cb = Qa[:, :nalpha], Qb[:, :nbeta]
    return 0.5 * np.vstack([Ca @ Ca.T, Cb @ Cb.T])


def basis_for(mol, name, pure=True):
    b = AOBasis.load(mol.atoms(), name)
    b.set_pure(pure)
    return b


def perturbed(D, norm, seed):
    rng = np.random.default_rng(seed)
    E = rng.standard_normal(D.shape)
    E = E + E.T
    return D + E * (norm / np.linalg.norm(E))
