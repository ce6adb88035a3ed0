"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run in a container that has the reference checkout, named by the MDTRAJ_REF
environment variable (the directory that holds the mdtraj/ package of the
reference project); never on the GPU host.  It builds the reference's
own Cython RMSD extension (mdtraj/rmsd/_rmsd.pyx with its C++ kernels) and
its XTC reader out of tree under oracle/_ref/py (git-ignored), imports them
through a stub ``mdtraj`` package, and records:

* frame0_xtc.npz  — examples/data/frame0.xtc (501 frames x 22 atoms) as read
                    by the reference reader, with the reference's md.rmsd to
                    frame 0 (plain, precentered, axis-major), its traces and
                    the FP64 Kabsch values.  The notebook pin
                    (examples/iterload.ipynb: max 0.18972313 nm at index 44,
                    from the lossless HDF5 copy) is stored for the test.
* alignment_6pt.npz — the 6-point known answer of tests/test_alignment.py:29-43
                    (read from the test file as text): a 90 degree rotation of
                    the set has RMSD 0.
* synthetic.npz   — small seeded cases (odd atom counts, exact copies,
                    degenerate 1-3 atom frames, atom_indices subsets,
                    superpose=False) with the reference's outputs.
* superpose_rmsf.npz — Trajectory.superpose (all atoms, a subset, another
                    reference object with shifted indices), rmsf (against
                    the trajectory itself, None, a subset, another reference,
                    with the in-place centring side effects) and
                    getMultipleAlignDisplaceRMSDs_atom_major (distances and
                    rotation matrices), all from the reference.
* xtc_{water,tiny,wide}.xtc + xtc_cases.npz — synthetic trajectories written
                    by the reference's XTC writer, with its reader's output
                    (coordinates, time, step, box) for the GPU decoder.
* center_mass.npz — Trajectory.center_coordinates(mass_weighted=True), run
                    from the reference's own source of that method and of
                    compute_center_of_mass.

Usage:  MDTRAJ_REF=<reference checkout> python tests/golden/make_golden.py [fixture ...]
"""
from __future__ import annotations

import ast
import os
import shutil
import subprocess
import sys
import types
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
if not os.environ.get("MDTRAJ_REF"):
    sys.exit("make_golden.py: set MDTRAJ_REF to the reference checkout (the directory holding mdtraj/)")
REF = Path(os.environ["MDTRAJ_REF"])
OUT = Path(__file__).resolve().parent
BUILD = REPO / "oracle" / "_ref" / "py"
SRC = REPO / "oracle" / "_ref" / "pysrc"

sys.path.insert(0, str(REPO))


def build_reference_python() -> None:
    """Cythonises the reference's _rmsd and xtc modules from a scratch copy."""
    if (BUILD / "mdtraj" / "_rmsd.done").exists():
        return
    if SRC.exists():
        shutil.rmtree(SRC)
    (SRC / "mdtraj" / "formats").mkdir(parents=True)
    shutil.copytree(REF / "mdtraj" / "rmsd", SRC / "mdtraj" / "rmsd")
    shutil.copytree(REF / "mdtraj" / "formats" / "xtc", SRC / "mdtraj" / "formats" / "xtc")
    for p in SRC.rglob("*"):
        p.chmod(0o755 if p.is_dir() else 0o644)
    setup = SRC / "setup_ref.py"
    setup.write_text(
        f"""
import numpy as np
from setuptools import setup, Extension
from Cython.Build import cythonize
R = "{SRC}/mdtraj/rmsd"
X = "{SRC}/mdtraj/formats/xtc"
simd = ["-msse2", "-mssse3"] if __import__("platform").machine() == "x86_64" else []
exts = [
    Extension("mdtraj._rmsd", [f"{{R}}/src/theobald_rmsd.cpp", f"{{R}}/src/rotation.cpp", f"{{R}}/src/center.cpp", f"{{R}}/_rmsd.pyx"],
              include_dirs=[f"{{R}}/include", np.get_include()], language="c++",
              extra_compile_args=["-fopenmp", "-O3", "-funroll-loops", "--std=c++11"] + simd, extra_link_args=["-fopenmp"]),
    Extension("mdtraj.formats.xtc", [f"{{X}}/src/xdrfile.c", f"{{X}}/src/xdr_seek.c", f"{{X}}/src/xdrfile_xtc.c", f"{{X}}/xtc.pyx"],
              include_dirs=[f"{{X}}/include", X, np.get_include()]),
]
setup(name="refbuild", ext_modules=cythonize(exts, language_level=3, force=True),
      script_args=["build_ext", "--build-lib", "{BUILD}", "--build-temp", "{SRC}/tmp"])
"""
    )
    subprocess.run([sys.executable, str(setup)], check=True, cwd=SRC, stdout=subprocess.DEVNULL)
    pkg = BUILD / "mdtraj"
    (pkg / "__init__.py").write_text("")
    (pkg / "formats" / "__init__.py").write_text("")
    shutil.copy(REF / "mdtraj" / "formats" / "registry.py", pkg / "formats" / "registry.py")
    if (pkg / "utils").exists():
        shutil.rmtree(pkg / "utils")
    shutil.copytree(REF / "mdtraj" / "utils", pkg / "utils")
    (pkg / "_rmsd.done").write_text("ok")


def import_reference():
    sys.path.insert(0, str(BUILD))
    from mdtraj import _rmsd  # noqa: E402
    from mdtraj.formats import xtc  # noqa: E402

    return _rmsd, xtc


class Traj:
    """Duck-typed stand-in for mdtraj.Trajectory (only .xyz and ._rmsd_traces
    are read by the reference's rmsd())."""

    def __init__(self, xyz):
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float32)
        self._rmsd_traces = None


def ref_rmsd(_rmsd, target, ref, frame=0, **kw):
    t = Traj(np.array(target, copy=True))
    r = t if ref is target else Traj(np.array(ref, copy=True))
    return np.asarray(_rmsd.rmsd(t, r, frame, **kw), dtype=np.float32)


def frame0_fixture(_rmsd, xtc) -> None:
    from oracle import fp64

    with xtc.XTCTrajectoryFile(str(REF / "examples" / "data" / "frame0.xtc")) as f:
        xyz, time, step, box = f.read()
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    t = Traj(xyz.copy())
    plain = np.asarray(_rmsd.rmsd(t, t, 0), dtype=np.float32)
    centred_after = t.xyz.copy()  # md.rmsd centres in place
    tc = Traj(xyz.copy())
    traces = np.asarray(_rmsd._center_inplace_atom_major(tc.xyz), dtype=np.float32)
    tc._rmsd_traces = traces
    pre = np.asarray(_rmsd.rmsd(tc, tc, 0, precentered=True), dtype=np.float32)
    axis = np.ascontiguousarray(tc.xyz.transpose(0, 2, 1))
    axis_rmsd = np.asarray(_rmsd.getMultipleRMSDs_axis_major(axis, axis, traces, traces, 0), dtype=np.float32)
    pre10 = np.asarray(_rmsd.rmsd(tc, tc, 10, precentered=True), dtype=np.float32)
    nosup = ref_rmsd(_rmsd, xyz, xyz, 0, superpose=False)
    sel = np.arange(3, 19)
    sel_rmsd = ref_rmsd(_rmsd, xyz, xyz, 0, atom_indices=sel)
    np.savez_compressed(
        OUT / "frame0_xtc.npz",
        xyz=xyz,
        rmsd_frame0=plain,
        xyz_after_rmsd=centred_after,
        traces=traces,
        centred=tc.xyz,
        rmsd_precentered_frame0=pre,
        rmsd_precentered_frame10=pre10,
        rmsd_axis_major_frame0=axis_rmsd,
        rmsd_nosuperpose_frame0=nosup,
        atom_indices=sel,
        rmsd_atom_indices_frame0=sel_rmsd,
        kabsch_fp64_frame0=fp64.kabsch_rmsd(xyz, xyz[0]),
        notebook_h5_max=np.float64(0.18972313),
        notebook_h5_argmax=np.int64(44),
    )
    print("frame0: max", plain.max(), "at", int(plain.argmax()), "first", plain[:5])


def alignment_fixture() -> None:
    src = (REF / "tests" / "test_alignment.py").read_text()
    tree = ast.parse(src)
    found = {}
    for node in tree.body:
        if isinstance(node, ast.Assign) and len(node.targets) == 1 and isinstance(node.targets[0], ast.Name):
            name = node.targets[0].id
            if name in ("xyz1", "rotation") and isinstance(node.value, ast.Call):
                found[name] = np.array(ast.literal_eval(node.value.args[0]), dtype=np.float64)
    xyz1, rot = found["xyz1"], found["rotation"]
    offset = np.array([0.25, -1.5, 0.75])
    xyz2 = rot.dot(xyz1.T).T + offset
    np.savez_compressed(OUT / "alignment_6pt.npz", xyz1=xyz1.astype(np.float32), xyz2=xyz2.astype(np.float32),
                        rotation=rot, expected_rmsd=np.float64(0.0), decimal=np.int64(5))


def synthetic_fixture(_rmsd) -> None:
    from mdtraj_gb300 import synth
    from oracle import fp64

    cases = {}
    # cfg0-like, odd atom count (not a multiple of 4), frame 0 is the reference
    ref, x = synth.single_reference_frames(64, 97, seed=11, sigma=0.05)
    cases["cfg0_small"] = (x, 0)
    # exact rotated/translated copies (true rmsd 0) and tiny noise
    ref, x = synth.single_reference_frames(32, 257, seed=12, sigma=np.array([0.0] * 16 + [1e-3] * 16))
    cases["copies"] = (x, 0)
    # degenerate structures: 1, 2, 3 atoms; 5 atoms
    for A in (1, 2, 3, 5):
        ref, x = synth.single_reference_frames(16, A, seed=20 + A, sigma=0.1)
        cases[f"atoms{A}"] = (x, 0)
    # larger frame count, frame != 0
    ref, x = synth.single_reference_frames(100, 1000, seed=13, sigma=0.05)
    cases["cfg0_mid"] = (x, 7)
    arrays = {}
    for name, (x, frame) in cases.items():
        arrays[f"{name}__xyz"] = x
        arrays[f"{name}__frame"] = np.int64(frame)
        arrays[f"{name}__ref"] = ref_rmsd(_rmsd, x, x, frame)
        arrays[f"{name}__fp64"] = fp64.kabsch_rmsd(x, x[frame])
        arrays[f"{name}__nosup"] = ref_rmsd(_rmsd, x, x, frame, superpose=False)
    # atom_indices / ref_atom_indices with a different reference object
    ref, x = synth.single_reference_frames(40, 120, seed=14, sigma=0.05)
    other = np.ascontiguousarray(np.concatenate([x[:5, 60:], x[:5, :60]], axis=1))
    ai = np.arange(0, 60)
    rai = np.arange(60, 120)
    arrays["indices__xyz"] = x
    arrays["indices__other"] = other
    arrays["indices__ai"] = ai
    arrays["indices__rai"] = rai
    arrays["indices__ref"] = np.asarray(
        _rmsd.rmsd(Traj(x.copy()), Traj(other.copy()), 2, atom_indices=ai, ref_atom_indices=rai), dtype=np.float32)
    np.savez_compressed(OUT / "synthetic.npz", **arrays)


def ref_superpose(_rmsd, xyz, ref_xyz, frame, ai=None, rai=None):
    """Trajectory.superpose (core/trajectory.py:1113-1165 is plain numpy around
    the compiled superpose_atom_major, and core/ is not importable here):
    centre on the alignment atoms' float64 mean, centre the reference frame,
    float32 traces, the compiled rotation, then add the reference offset."""
    ai = slice(None) if ai is None else ai
    rai = ai if rai is None else rai
    x = np.array(xyz, dtype=np.float32, copy=True, order="C")
    align = np.asarray(x[:, ai, :], order="c")
    ref_align = np.array(ref_xyz[frame, rai, :], dtype=np.float32, copy=True, order="c").reshape(1, -1, 3)
    offset = np.mean(align, axis=1, dtype=np.float64).reshape(len(x), 1, 3)
    align -= offset
    if align.ctypes.data != x.ctypes.data:
        x -= offset
    ref_offset = ref_align[0].astype("float64").mean(0)
    ref_align[0] -= ref_offset
    g = np.einsum("ijk,ijk->i", align, align)
    ref_g = np.einsum("ijk,ijk->i", ref_align, ref_align)
    _rmsd.superpose_atom_major(ref_align, align, ref_g, g, x, 0)
    x += ref_offset
    return x


def superpose_fixture(_rmsd) -> None:
    """superpose_rmsf.npz: Trajectory.superpose, rmsf and
    getMultipleAlignDisplaceRMSDs_atom_major from the reference."""
    from mdtraj_gb300 import synth

    ref, x = synth.single_reference_frames(30, 45, seed=31, sigma=0.2)
    # another reference object: noisy, rotated, translated copies of frames
    # 0-5 (atom k corresponds to atom k), and the same rolled by one atom
    # (atom k + 1 corresponds to atom k, for shifted reference indices)
    rng = np.random.default_rng(32)
    rot = synth.haar_rotations(6, rng)
    other = (np.einsum("fkj,fij->fki", x[:6].astype(np.float64) + rng.normal(size=(6, 45, 3)) * 0.05, rot)
             + rng.uniform(-2, 2, size=(6, 1, 3))).astype(np.float32)
    rolled = np.ascontiguousarray(np.roll(other, 1, axis=1))
    # selections of 16 atoms: the reference's vectorised msd_atom_major reads
    # whole 4-atom groups, so with a selection whose size is not a multiple of
    # 4 it reads past the end of the selected reference frame (rmsf and
    # superpose_atom_major pass the selection size as the padded size) and its
    # results change from call to call
    sub = np.arange(0, 32, 2)
    shifted = sub + 1
    arrays = {"xyz": x, "other": other, "rolled": rolled, "sub": sub, "shifted": shifted}
    arrays["sup_all_f3"] = ref_superpose(_rmsd, x, x, 3)
    arrays["sup_sub_f0"] = ref_superpose(_rmsd, x, x, 0, sub)
    arrays["sup_other_f2"] = ref_superpose(_rmsd, x, rolled, 2, sub, shifted)
    # rmsf: each call centres its target (and the reference frame) in place
    t = Traj(x.copy())
    arrays["rmsf_self_f0"] = np.asarray(_rmsd.rmsf(t, t, 0), dtype=np.float32)
    arrays["rmsf_self_f0_centred"] = t.xyz.copy()
    t = Traj(x.copy())
    arrays["rmsf_none"] = np.asarray(_rmsd.rmsf(t, None), dtype=np.float32)
    # with an explicit atom_indices the reference's rmsf() returns values that
    # change from call to call under OpenMP (measured here: the first atoms of
    # the selection differ between runs and from the serial result); the pin
    # for that case is the reference's own kernels composed along rmsf's data
    # flow (_rmsd.pyx:389-418): centre a copy of the selection and the selected
    # reference frame, rotate the uncentred selection about the origin
    t = Traj(x.copy())
    _rmsd.rmsf(t, Traj(x.copy()), 5, atom_indices=sub)
    arrays["rmsf_sub_f5_xyz_after"] = t.xyz.copy()
    sel = np.ascontiguousarray(x[:, sub])
    g_sel = np.asarray(_rmsd._center_inplace_atom_major(sel), dtype=np.float32)
    ref_sel = np.ascontiguousarray(x[5, sub])[None].copy()
    g_ref = np.asarray(_rmsd._center_inplace_atom_major(ref_sel), dtype=np.float32)
    disp = np.ascontiguousarray(x[:, sub]).copy()
    _rmsd.superpose_atom_major(ref_sel, sel, g_ref, g_sel, disp, 0, parallel=False)
    d = disp.astype(np.float64)
    arrays["rmsf_sub_f5"] = np.sqrt(((d - d.mean(0)) ** 2).sum(2).mean(0)).astype(np.float32)
    t = Traj(x.copy())
    r = Traj(other.copy())
    arrays["rmsf_other_f1"] = np.asarray(_rmsd.rmsf(t, r, 1), dtype=np.float32)
    arrays["rmsf_other_f1_ref_after"] = r.xyz.copy()
    # align-displace on padded, pre-centred alignment atoms
    n_al, n_di = 21, 30
    al = np.zeros((30, 24, 3), np.float32)
    al[:, :n_al] = x[:, :n_al] - x[:, :n_al].astype(np.float64).mean(1, keepdims=True)
    di = np.zeros((30, 32, 3), np.float32)
    di[:, :n_di] = x[:, 15:45]
    g = np.einsum("ijk,ijk->i", al, al).astype(np.float32)
    d, rot = _rmsd.getMultipleAlignDisplaceRMSDs_atom_major(al, al, g, g, di, di, n_al, n_di, 4)
    arrays.update(ad_align=al, ad_displ=di, ad_g=g, ad_rmsd=np.asarray(d, np.float32), ad_rot=np.asarray(rot, np.float32))
    np.savez_compressed(OUT / "superpose_rmsf.npz", **arrays)


def xtc_fixture(xtc) -> None:
    """xtc_*.xtc + xtc_cases.npz: synthetic trajectories written by the
    reference's XTC writer and read back by its reader (formats/xtc), for the
    GPU decoder.  Cases: 'water' (333 three-atom clusters + 2 atoms: runs of
    small integer differences), 'tiny' (7 atoms: stored uncompressed),
    'wide' (coordinates spanning 18,000 nm: per-dimension integer sizes)."""
    rng = np.random.default_rng(41)
    cases = {}
    centres = rng.uniform(0, 5, size=(333, 1, 3))
    offsets = rng.normal(0, 0.08, size=(333, 3, 3))
    base = np.concatenate([(centres + offsets).reshape(-1, 3), rng.uniform(0, 5, size=(2, 3))])
    cases["water"] = base[None] + rng.normal(0, 0.02, size=(40, len(base), 3))
    cases["tiny"] = rng.uniform(-1, 1, size=(12, 7, 3))
    wide = rng.uniform(-1, 1, size=(5, 50, 3))
    wide[:, :, 0] *= 9000.0
    cases["wide"] = wide
    arrays = {}
    for name, x in cases.items():
        x = x.astype(np.float32)
        n = len(x)
        path = OUT / f"xtc_{name}.xtc"
        time = (np.arange(n) * 2.5 + 10).astype(np.float32)
        step = (np.arange(n) * 1000 + 7).astype(np.int32)
        box = np.repeat((np.eye(3) * np.float32(5.5 + 0.1 * len(name)))[None], n, 0).astype(np.float32)
        with xtc.XTCTrajectoryFile(str(path), "w") as f:
            f.write(x, time=time, step=step, box=box)
        with xtc.XTCTrajectoryFile(str(path)) as f:
            xyz, t, st, bx = f.read()
        arrays[f"{name}__xyz"] = np.asarray(xyz, dtype=np.float32)
        arrays[f"{name}__time"] = np.asarray(t, dtype=np.float32)
        arrays[f"{name}__step"] = np.asarray(st, dtype=np.int32)
        arrays[f"{name}__box"] = np.asarray(bx, dtype=np.float32)
    np.savez_compressed(OUT / "xtc_cases.npz", **arrays)


def _reference_function(path: Path, name: str, cls: str | None = None):
    """Source of one function (or method of class `cls`) of a reference
    module, parsed with ast (core/ and geometry/ import compiled modules that
    are not built here, so the module itself cannot be imported)."""
    tree = ast.parse(path.read_text())
    body = tree.body
    if cls is not None:
        body = next(n for n in body if isinstance(n, ast.ClassDef) and n.name == cls).body
    node = next(n for n in body if isinstance(n, ast.FunctionDef) and n.name == name)
    node.decorator_list = []
    return ast.unparse(node)


def center_mass_fixture() -> None:
    """center_mass.npz: Trajectory.center_coordinates(mass_weighted=True) of
    the reference (core/trajectory.py:2114-2137 with
    geometry/distance.py:349-384, both run from their own source) on
    duck-typed trajectories whose atoms carry element masses.  Cases: 'mixed'
    (H/C/N/O/S masses), 'chunk' (2,101 atoms), 'hydrogen' (equal masses, the
    reference's test_center), 'nonfinite' (an inf and a NaN coordinate)."""
    ns = {"np": np}
    exec(_reference_function(REF / "mdtraj" / "geometry" / "distance.py", "compute_center_of_mass"), ns)
    meth = {"np": np, "distance": types.SimpleNamespace(compute_center_of_mass=ns["compute_center_of_mass"])}
    exec(_reference_function(REF / "mdtraj" / "core" / "trajectory.py", "center_coordinates", "Trajectory"), meth)

    class Atom:
        def __init__(self, mass):
            self.element = types.SimpleNamespace(mass=float(mass))

    class Top:
        def __init__(self, masses):
            self._atoms = [Atom(m) for m in masses]

        @property
        def atoms(self):
            return iter(self._atoms)

    class T:
        def __init__(self, xyz, masses):
            self.top = self.topology = Top(masses)
            self._xyz = xyz
            self._rmsd_traces = np.zeros(len(xyz), np.float32)

        @property
        def xyz(self):
            return self._xyz

        @xyz.setter
        def xyz(self, v):  # the reference setter's effect on these arrays (core/trajectory.py:1010-1029)
            self._xyz = np.asarray(v, dtype=np.float32)
            self._rmsd_traces = None

        @property
        def n_frames(self):
            return len(self._xyz)

    rng = np.random.default_rng(77)
    table = np.array([1.008, 12.011, 14.007, 15.999, 32.06])
    cases = {
        "mixed": (rng.uniform(-3, 5, size=(7, 23, 3)), table[rng.integers(0, 5, 23)]),
        "chunk": (rng.uniform(-1, 9, size=(3, 2101, 3)) + 40.0, table[rng.integers(0, 5, 2101)]),
        "hydrogen": (rng.normal(1.5, 2.0, size=(5, 37, 3)), np.full(37, 1.008)),
    }
    bad = rng.uniform(-2, 2, size=(3, 5, 3))
    bad[1, 2, 0] = np.inf
    bad[2, 4, 1] = np.nan
    cases["nonfinite"] = (bad, table[rng.integers(0, 5, 5)])
    arrays = {}
    for name, (x, masses) in cases.items():
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = T(x.copy(), masses)
        with np.errstate(invalid="ignore"):
            meth["center_coordinates"](t, mass_weighted=True)
        assert t._rmsd_traces is None
        arrays[f"{name}__xyz"] = x
        arrays[f"{name}__masses"] = masses
        arrays[f"{name}__centred"] = t.xyz
    np.savez_compressed(OUT / "center_mass.npz", **arrays)


FIXTURES = ("frame0", "alignment", "synthetic", "superpose", "xtc", "center_mass")


def main(only: list[str]) -> None:
    """Writes every fixture, or only those named on the command line."""
    want = set(only or FIXTURES)
    unknown = want - set(FIXTURES)
    if unknown:
        sys.exit(f"make_golden.py: unknown fixtures {sorted(unknown)}; choose from {FIXTURES}")
    build_reference_python()
    _rmsd, xtc = import_reference()
    if "frame0" in want:
        frame0_fixture(_rmsd, xtc)
    if "alignment" in want:
        alignment_fixture()
    if "synthetic" in want:
        synthetic_fixture(_rmsd)
    if "superpose" in want:
        superpose_fixture(_rmsd)
    if "xtc" in want:
        xtc_fixture(xtc)
    if "center_mass" in want:
        center_mass_fixture()
    for p in sorted(OUT.glob("*.npz")):
        print(p.name, p.stat().st_size, "bytes")


if __name__ == "__main__":
    main(sys.argv[1:])
