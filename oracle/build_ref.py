"""Recipe: compile the reference project's own CUDA kernels into oracle/_ref/ (TEST INFRASTRUCTURE).

The reference keeps each kernel as a ``.cu`` text file and compiles it at run
time with NVRTC after two text substitutions (``sources/sim_state.py:260-263``,
``sources/wave_packet.py:107-110``, ``sources/measurement.py:104-107``):
``PATH_TO_SOURCES`` becomes the absolute path of its ``sources`` folder and
``T_WF_FLOAT`` becomes ``float`` or ``double`` (which also turns
``T_WF_FLOAT3`` into ``float3``/``double3``). This recipe makes the same two
substitutions on the files where they lie in the reference tree, supplies a
project-written ``complex<T>`` (``oracle/ref_shim/cupy/complex.cuh``) in place
of CuPy's ``<cupy/complex.cuh>`` (``sources/cuda_kernels/common.cu:4``), and
compiles each kernel unchanged with nvcc for sm_103a into a device-only
fatbinary under ``oracle/_ref/``. Template kernels, which the reference
instantiates through ``cp.RawModule(name_expressions=...)``
(``sources/measurement.py:123-128``, ``:340-345``), get one explicit
instantiation per sample box in a generated wrapper.

Nothing here is product code: ``oracle/ref_gpu.py`` loads the fatbinaries
through the CUDA driver API for the parity tests. The substituted sources are
written to a temporary folder and deleted; only the fatbinaries are kept, and
``oracle/_ref/`` is git-ignored.

Usage: ``python oracle/build_ref.py [REFERENCE_ROOT]`` (default: the
reference checkout at /root/reference). Without a reference checkout the
recipe does nothing and reports that it skipped.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SHIM = HERE / "ref_shim"
DEFAULT_REFERENCE = "/root/reference"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (reference file, kernel symbol, precisions). "-" marks a file without T_WF_FLOAT.
PLAIN_KERNELS = [
    ("kinetic_operator.cu", "kinetic_operator_kernel", ("float", "double")),
    ("potential_operator.cu", "potential_operator_kernel", ("float", "double")),
    ("power_series_operator.cu", "next_s", ("float",)),
    ("gaussian_wave_packet.cu", "wave_packet_kernel", ("float", "double")),
    ("potential_wall.cu", "potential_wall_kernel", ("-",)),
    ("absorbing_potential.cu", "absorbing_potential_kernel", ("-",)),
]


def _box(bottom_voxel, count, n):
    return tuple(int(c) for c in count) + tuple(int(v) for v in n)


def template_boxes():
    """Sample boxes (sample counts + grid shape) the parity tests observe with the
    reference's template kernels: the fixture grid's boxes, config 1's whole grid and
    config 3's transmitted box P(x > 1) and observation box."""
    sys.path.insert(0, str(HERE.parent))
    from oracle import wfs_oracle as orc

    boxes = set()
    for count, n in FIXTURE_BOXES:
        boxes.add(_box(None, count, n))
    boxes.add(_box(None, (63, 63, 63), (64, 64, 64)))
    n3 = (256, 256, 256)
    inner = 40.0 - 16 * (80.0 / 256)
    _, cnt = orc.simpson_box_from_corners((1.0, -inner, -inner), (inner, inner, inner), (80.0,) * 3, n3)
    boxes.add(_box(None, cnt, n3))
    _, cnt = orc.simpson_box_from_corners((-inner,) * 3, (inner,) * 3, (80.0,) * 3, n3)
    boxes.add(_box(None, cnt, n3))
    return sorted(boxes)


# Boxes on the fixture grid (32, 24, 16): sample counts and grid shape.
FIXTURE_GRID = (32, 24, 16)
FIXTURE_BOXES = [((21, 15, 11), FIXTURE_GRID), ((29, 21, 13), FIXTURE_GRID), ((31, 23, 15), FIXTURE_GRID)]


def fatbin_name(stem, precision, box=None):
    tag = {"float": "f32", "double": "f64", "-": "f32"}[precision]
    name = f"{stem}_{tag}"
    if box is not None:
        name += "_" + "_".join(str(v) for v in box)
    return name + ".fatbin"


def _substitute(text, sources_dir, precision):
    text = text.replace("PATH_TO_SOURCES", sources_dir)
    if precision != "-":
        text = text.replace("T_WF_FLOAT", precision)
    return text


def _nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return exe


def _compile(src: Path, out: Path):
    cmd = [_nvcc(), *ARCH, "-std=c++17", "-O3", "-fatbin", "-I", str(SHIM), "-diag-suppress", "177,550",
           str(src), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return out


def jobs(reference_root: Path, tmp: Path):
    """(substituted source, fatbin path) pairs for every kernel and instantiation."""
    kdir = reference_root / "sources" / "cuda_kernels"
    sources_dir = str((reference_root / "sources").resolve())
    out = []
    for fname, _sym, precisions in PLAIN_KERNELS:
        text = (kdir / fname).read_text()
        for p in precisions:
            src = tmp / fatbin_name(Path(fname).stem, p).replace(".fatbin", ".cu")
            src.write_text(_substitute(text, sources_dir, p))
            out.append((src, OUT / fatbin_name(Path(fname).stem, p)))
    for fname, sym, ctype, itype in (("volume_probability.cu", "volume_probability_kernel", "unsigned int", "u"),
                                     ("expected_location.cu", "expected_location_kernel", "int", "i")):
        text = (kdir / fname).read_text()
        for p in ("float", "double"):
            base = _substitute(text, sources_dir, p)
            for box in template_boxes():
                c, n = box[:3], box[3:]
                args = ", ".join([f"{v}u" for v in c] + [f"{v}u" if itype == "u" else f"{v}" for v in n])
                if fname.startswith("volume"):
                    sig = f"complex<{p}>*, {p}*, {p}, {p}, {p}, unsigned int, unsigned int, unsigned int"
                else:
                    sig = f"complex<{p}>*, {p}*, {p}*, {p}, {p}, {p}, int, int, int"
                inst = f"\ntemplate __global__ void {sym}<{args}>({sig});\n"
                src = tmp / fatbin_name(Path(fname).stem, p, box).replace(".fatbin", ".cu")
                src.write_text(base + inst)
                out.append((src, OUT / fatbin_name(Path(fname).stem, p, box)))
    return out


def build(reference_root=None, verbose=False) -> bool:
    """Compile every reference kernel; returns False (and builds nothing) without a
    reference checkout. Skips the work when every fatbinary is newer than this recipe
    and the shim header."""
    root = Path(reference_root or os.environ.get("WFS_REFERENCE_ROOT", DEFAULT_REFERENCE))
    kdir = root / "sources" / "cuda_kernels"
    if not kdir.is_dir():
        if verbose:
            print(f"reference kernels not found under {root}: oracle/_ref not rebuilt", file=sys.stderr)
        return False
    OUT.mkdir(exist_ok=True)
    newest_input = max(p.stat().st_mtime for p in [Path(__file__), SHIM / "cupy" / "complex.cuh",
                                                     *kdir.glob("*.cu")])
    with tempfile.TemporaryDirectory(prefix="wfs_ref_") as td:
        todo = [(s, o) for s, o in jobs(root, Path(td))
                if not o.exists() or o.stat().st_mtime < newest_input]
        workers = max(2, min(len(todo), os.cpu_count() or 2))
        if todo:
            with cf.ThreadPoolExecutor(workers) as ex:
                list(ex.map(lambda so: _compile(*so), todo))
    if verbose:
        print(f"reference kernels: {len(todo)} fatbinaries rebuilt in {OUT}", file=sys.stderr)
    return True


if __name__ == "__main__":
    ok = build(sys.argv[1] if len(sys.argv) > 1 else None, verbose=True)
    sys.exit(0 if ok else 0)
