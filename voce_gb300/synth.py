"""Synthetic microstructures and inputs in the Voce reference's file formats.

The reference reads three inputs (no generator ships with it; its 64^3 mesh
``mesh_64_rand_125.txt`` is missing from the reference tree):

* the namelist parsed by ``GetNameList`` (reference io.c:25-122): lines
  ``key v1 v2 ...``, ``#`` comments, case-sensitive keys, unknown keys
  silently ignored;
* the single-crystal ``.sx`` file read at fixed line positions by
  ``PlasticInit`` (reference init.c:51-186);
* the mesh read by ``InitMicroStruct`` (reference init.c:410-433): one line
  per voxel, ``phi1 Phi phi2 i j k grain phase`` (Bunge angles in degrees,
  1-based indices, x slowest / z fastest), each line under 80 characters
  because the reader uses ``fgets(buffer, 80, fp)``.

Angles are written with ``%.6f`` and the in-memory arrays hold the value a
correctly rounded parse of that text gives, so a run that reads the text
file and a run that is handed the arrays see identical doubles.
"""
from __future__ import annotations

import dataclasses
import hashlib
import os
from typing import Dict, Optional, Sequence

import numpy as np

# 12 {111}<110> systems, slip-plane normal n then direction b, in the order
# of the reference's Cu_p.sx:24-35 (crystal frame, unnormalised integers).
FCC_111_110 = (
    ((1, 1, -1), (0, 1, 1)), ((1, 1, -1), (1, 0, 1)), ((1, 1, -1), (1, -1, 0)),
    ((1, -1, -1), (0, 1, -1)), ((1, -1, -1), (1, 0, 1)), ((1, -1, -1), (1, 1, 0)),
    ((1, -1, 1), (0, 1, 1)), ((1, -1, 1), (1, 0, -1)), ((1, -1, 1), (1, 1, 0)),
    ((1, 1, 1), (0, 1, -1)), ((1, 1, 1), (1, 0, -1)), ((1, 1, 1), (1, -1, 0)),
)


@dataclasses.dataclass
class Material:
    """Cubic elastic constants (MPa) plus one slip mode (power law + Voce)."""
    c11: float = 168400.0
    c12: float = 121400.0
    c44: float = 75400.0
    nu: float = 0.35
    nrs: float = 20.0        # rate-sensitivity exponent n
    gamd0: float = 1e-3      # reference shear rate
    tau0f: float = 12.0
    tau0b: float = 12.0
    tau1: float = 6.0
    thet0: float = 200.0
    thet1: float = 3.0
    latent: Dict[str, float] = dataclasses.field(default_factory=lambda: {
        "self": 1.0, "coplane": 1.0, "cross": 1.0, "glissile": 1.0,
        "Hirth": 1.0, "lomer": 1.0})
    slip: Sequence = FCC_111_110


CU_LIKE = Material()


@dataclasses.dataclass
class Load:
    """Velocity-gradient / stress boundary conditions in Voigt order
    11,22,33,23,13,12 (reference io.c:37-40, init.c:713-745)."""
    velgrad_flag: Sequence[int]
    velgrad: Sequence[float]
    stress_flag: Sequence[int]
    stress: Sequence[float] = (0.0,) * 6


def tension_z(rate: float = 1e-3) -> Load:
    """Uniaxial tension along z with the lateral normal stresses held at 0."""
    return Load((0, 0, 1, 1, 1, 1), (-0.5 * rate, -0.5 * rate, rate, 0, 0, 0),
                (1, 1, 0, 0, 0, 0))


def plane_strain_compression(rate: float = 1e-3) -> Load:
    """All six velocity-gradient components known: Lxx=+rate, Lzz=-rate."""
    return Load((1, 1, 1, 1, 1, 1), (rate, 0.0, -rate, 0.0, 0.0, 0.0),
                (0, 0, 0, 0, 0, 0))


def random_traceless_load(rng: np.random.Generator, rate: float = 1e-3) -> Load:
    """Random symmetric traceless velocity gradient of Frobenius norm `rate`.

    The reference's velocity-gradient BC is 6-component Voigt, so it is always
    symmetric (reference init.c:716 VoigtToFull); all six components known."""
    a = rng.standard_normal((3, 3))
    s = 0.5 * (a + a.T)
    s -= np.eye(3) * np.trace(s) / 3.0
    s *= rate / np.linalg.norm(s)
    # quantised to 1e-6 so that a namelist line fits the reader's 80 bytes;
    # L33 is set so that the trace stays zero after rounding
    v = [round(float(x), 6) for x in (s[0, 0], s[1, 1], s[2, 2], s[1, 2], s[0, 2], s[0, 1])]
    v[2] = round(-(v[0] + v[1]), 6)
    return Load((1,) * 6, tuple(v), (0,) * 6)


@dataclasses.dataclass
class Mesh:
    dims: tuple
    euler_deg: np.ndarray   # (nvox, 3) float64, exactly the %.6f-parsed values
    grain: np.ndarray       # (nvox,) int32, 1-based
    phase: np.ndarray       # (nvox,) int32, 1-based

    @property
    def nvox(self) -> int:
        return int(np.prod(self.dims))

    def digest(self) -> str:
        h = hashlib.sha256()
        h.update(np.ascontiguousarray(self.euler_deg, dtype="<f8").tobytes())
        h.update(np.ascontiguousarray(self.grain, dtype="<i4").tobytes())
        h.update(np.ascontiguousarray(self.phase, dtype="<i4").tobytes())
        return h.hexdigest()[:16]


def _quantize_deg(a: np.ndarray) -> np.ndarray:
    """Round to the value that parsing the '%.6f' text of `a` gives."""
    txt = np.char.mod("%.6f", a.ravel())
    return txt.astype(np.float64).reshape(a.shape)


def so3_uniform_bunge(rng: np.random.Generator, n: int) -> np.ndarray:
    """n orientations uniform on SO(3) as Bunge angles in degrees:
    phi1 = 360 u1, Phi = acos(2 u2 - 1), phi2 = 360 u3."""
    u = rng.random((n, 3))
    e = np.empty((n, 3))
    e[:, 0] = 360.0 * u[:, 0]
    e[:, 1] = np.degrees(np.arccos(2.0 * u[:, 1] - 1.0))
    e[:, 2] = 360.0 * u[:, 2]
    return _quantize_deg(e)


def voxel_grains_mesh(n: int, seed: int) -> Mesh:
    """Every voxel its own grain (grain id = voxel index + 1)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nvox = n ** 3
    eul = so3_uniform_bunge(rng, nvox)
    return Mesh((n, n, n), eul, np.arange(1, nvox + 1, dtype=np.int32),
                np.ones(nvox, dtype=np.int32))


def voronoi_labels(n: int, seeds: np.ndarray) -> np.ndarray:
    """Periodic Voronoi labels (0-based) of the voxel centres (i+0.5)/n of an
    n^3 grid, minimum-image distance.  Uses a periodic KD-tree when scipy is
    present, else a chunked brute force (ties: lowest id)."""
    g = (np.arange(n) + 0.5) / n
    try:
        from scipy.spatial import cKDTree
        tree = cKDTree(np.mod(seeds, 1.0), boxsize=1.0)
        lab = np.empty(n ** 3, dtype=np.int32)
        yz = np.stack(np.meshgrid(g, g, indexing="ij"), -1).reshape(-1, 2)
        for x in range(n):
            pts = np.empty((n * n, 3))
            pts[:, 0] = g[x]
            pts[:, 1:] = yz
            _, idx = tree.query(pts, k=1)
            lab[x * n * n:(x + 1) * n * n] = idx
        return lab
    except ImportError:
        pass
    lab = np.empty(n ** 3, dtype=np.int32)
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    for s in range(0, pts.shape[0], 4096):
        d = pts[s:s + 4096, None, :] - seeds[None, :, :]
        d -= np.round(d)
        lab[s:s + 4096] = np.argmin((d * d).sum(-1), axis=1)
    return lab


def voronoi_mesh(n: int, n_grains: int, seed: int) -> Mesh:
    """Periodic Voronoi tessellation of n^3 voxels into n_grains grains with
    seeds uniform in the unit cube, one SO(3)-uniform orientation per grain.
    The generator draws the seeds first, then the orientations."""
    rng = np.random.Generator(np.random.PCG64(seed))
    seeds = rng.random((n_grains, 3))
    eul_g = so3_uniform_bunge(rng, n_grains)
    lab = voronoi_labels(n, seeds)
    return Mesh((n, n, n), eul_g[lab], (lab + 1).astype(np.int32),
                np.ones(n ** 3, dtype=np.int32))


def voronoi_mesh_box(dims, n_grains: int, seed: int) -> Mesh:
    """voronoi_mesh on an nx x ny x nz grid: voxel centres ((i+0.5)/nx,
    (j+0.5)/ny, (k+0.5)/nz) in the periodic unit cube, brute-force labels
    (ties: lowest id).  For small grids."""
    nx, ny, nz = dims
    rng = np.random.Generator(np.random.PCG64(seed))
    seeds = rng.random((n_grains, 3))
    eul_g = so3_uniform_bunge(rng, n_grains)
    axes = [(np.arange(m) + 0.5) / m for m in (nx, ny, nz)]
    pts = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
    d = pts[:, None, :] - seeds[None, :, :]
    d -= np.round(d)
    lab = np.argmin((d * d).sum(-1), axis=1).astype(np.int32)
    return Mesh((nx, ny, nz), eul_g[lab], lab + 1, np.ones(nx * ny * nz, dtype=np.int32))


def write_mesh(path: str, mesh: Mesh) -> None:
    nx, ny, nz = mesh.dims
    ii, jj, kk = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1),
                             np.arange(1, nz + 1), indexing="ij")
    cols = np.column_stack([mesh.euler_deg, ii.ravel(), jj.ravel(), kk.ravel(),
                            mesh.grain, mesh.phase])
    np.savetxt(path, cols, fmt="%.6f %.6f %.6f %d %d %d %d %d")


def write_sx(path: str, mat: Material) -> None:
    """One-mode .sx in the line layout PlasticInit reads (init.c:65-178)."""
    lines = [
        "# Crystal system (XtalSys):", "CUBIC", "",
        "# Crystal axes (XtalAxis):", "1.0 1.0 1.0", "",
        "# Total number of modes listed in the file (N_modes_max):", "1", "",
        "# Number of modes to be used in the calculation (N_modes):", "1", "",
        "# Labels of the modes to be used (iMode):", "1", "",
        "# Mode# 1 -- <110>(111) SLIP",
        "\tnsmx\tnrsx\tgamd0x\ttwshx\tisectwx",
        "\t%d\t\t%.17g\t\t%.17g\t\t0.0\t\t0" % (len(mat.slip), mat.nrs, mat.gamd0),
        "\ttau0xf\ttau0xb\ttau1x\tthet0\tthet1",
        "\t%.17g\t\t%.17g\t\t%.17g\t\t%.17g\t\t%.17g" % (
            mat.tau0f, mat.tau0b, mat.tau1, mat.thet0, mat.thet1),
        "\thselfx\thlatex2", "\t1.0\t1.0", "\tSlip (n-b)",
    ]
    for n_, b_ in mat.slip:
        lines.append("\t%d %d %d\t\t%d %d %d" % (*n_, *b_))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_namelist(path: str, dims, mat: Material, load: Load, *,
                   time_step: float, n_steps: int, err: float = 1e-5,
                   iter_max: int = 200, print_control=(0, 1),
                   update_flag: int = 1, hard_flag: int = 1, tex_flag: int = 0,
                   sx_name: str = "mat.sx", mesh_name: str = "mesh.txt",
                   n_phases: int = 2) -> None:
    """Namelist with every key GetNameList knows (io.c:25-52).  The latent
    hardening keys are written as given; the Hirth coefficient is written as
    ``Hirth`` -- the capitalisation the reference's own example input uses
    (input:86) -- which the case-sensitive parser ignores, so the effective
    Hirth coefficient is 0, exactly as in the reference."""
    f6 = lambda v: " ".join(repr(float(x)) for x in v)   # shortest round trip
    i6 = lambda v: " ".join("%d" % x for x in v)
    L = [
        "# generated", "N_phases\t%d" % n_phases,
        "CellDim\t\t%d %d %d" % tuple(dims),
        "initial_ms\t\t%s" % mesh_name,
        "Type_phases\t\t0  1",
        "ElastConst_PhaseI\t%s" % f6((mat.c11, mat.c12, mat.c44, mat.nu)),
        "Slip_PhaseI\t\t%s" % sx_name,
        "ElastConst_PhaseII\t0.0 0.0 0.0 0.0",
        "Slip_PhaseII\tXXXXX",
        "VelGrad_BC_Flag\t\t%s" % i6(load.velgrad_flag),
        "VelGrad_BC\t\t%s" % f6(load.velgrad),
        "Stress_BC_Flag\t\t%s" % i6(load.stress_flag),
        "Stress_BC\t%s" % f6(load.stress),
        "TimeStep\t%r" % float(time_step),
        "N_steps\t\t%d" % n_steps,
        "Err\t\t%r" % float(err),
        "IterMax\t\t%d" % iter_max,
        "PrintControl\t%d\t%d" % tuple(print_control),
        "Update_Flag\t\t%d" % update_flag,
        "Hard_Flag\t\t%d" % hard_flag,
        "Tex_Flag\t\t%d" % tex_flag,
    ]
    for k in ("self", "coplane", "cross", "glissile", "Hirth", "lomer"):
        L.append("%s\t%r\t0.0" % (k, float(mat.latent[k])))
    for s in L:
        assert len(s) < 79, s
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


@dataclasses.dataclass
class Case:
    """One RVE job: mesh + material + load + time stepping."""
    name: str
    mesh: Mesh
    mat: Material
    load: Load
    time_step: float
    n_steps: int
    err: float = 1e-5
    iter_max: int = 200
    update_flag: int = 1
    hard_flag: int = 1

    def write(self, d: str, print_control=(0, 1), tex_flag: int = 0) -> str:
        """Write namelist, .sx and mesh into directory d; return the namelist
        path.  File names are relative (the reference's namelist lines are
        read into 80-byte buffers)."""
        os.makedirs(d, exist_ok=True)
        write_mesh(os.path.join(d, "mesh.txt"), self.mesh)
        write_sx(os.path.join(d, "mat.sx"), self.mat)
        nl = os.path.join(d, "input")
        write_namelist(nl, self.mesh.dims, self.mat, self.load,
                       time_step=self.time_step, n_steps=self.n_steps,
                       err=self.err, iter_max=self.iter_max,
                       print_control=print_control, tex_flag=tex_flag,
                       update_flag=self.update_flag, hard_flag=self.hard_flag)
        return nl


def config1(n_steps: int = 50) -> Case:
    """16^3, one grain per voxel, Cu-like, tension z, 50 x 2e-4."""
    return Case("cfg1_16", voxel_grains_mesh(16, 1), CU_LIKE, tension_z(),
                0.2, n_steps)


def config2(n_steps: int = 100) -> Case:
    """64^3, 125 periodic Voronoi grains, tension z, 100 x 2e-4."""
    return Case("cfg2_64", voronoi_mesh(64, 125, 2), CU_LIKE, tension_z(),
                0.2, n_steps)


def config3(n_steps: int = 250) -> Case:
    """256^3, 4096 periodic Voronoi grains, plane-strain compression."""
    return Case("cfg3_256", voronoi_mesh(256, 4096, 3), CU_LIKE,
                plane_strain_compression(), 0.2, n_steps)


def small_case(n: int, n_grains: int, seed: int, n_steps: int,
               load: Optional[Load] = None, time_step: float = 0.2) -> Case:
    """A small Voronoi case for parity tests."""
    return Case("small_%d_%d_%d" % (n, n_grains, seed),
                voronoi_mesh(n, n_grains, seed), CU_LIKE,
                load or tension_z(), time_step, n_steps)
