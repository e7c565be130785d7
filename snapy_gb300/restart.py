"""Restart files: the block parts, the bundle that combines them, the
reader and its metadata checks, as the reference writes and reads them.

Reference: RestartOutput::write_output_file / combine_blocks /
make_restart_bundle, load_restart and check_restart_metadata
(src/output/restart.cpp:40-350), src/output/restart_metadata.hpp, and the
resume MeshBlockImpl::_init_from_restart (src/mesh/meshblock_restart.cpp
:33-236).

Layout on disk.
* One part per block, ``<basename>.block<rank>.<number>.part`` (``final`` in
  place of the number for the last write): a dict of named CPU tensors.
* Combined: with one part, the part renamed ``<basename>.<number>.restart``;
  with several, a bundle of that name -- the magic line
  ``SNAPY_RESTART_BUNDLE_V1``, the part count, one ``<part name>\\t<bytes>``
  line per part, an empty line, then the parts' bytes in index order -- and
  the parts removed.
* A part's tensors: hydro_u (the conserved TOTALS), last_time, last_cycle,
  file_number / next_time (the output schedule, one entry here: the restart
  output itself), scalar_s when tracers are carried, and for an FP32 block
  stored as anomalies about an FP64 hydrostatic base: hydro_u_stored (the
  anomaly bits, so a resume continues bit for bit), hydro_ref (the base:
  rho_b | p_b | e_b | pf_b | r_b, nc1 each and one more face), the metadata
  [version 1, stored bits] and the grid faces hydro_ref_x1f/x2f/x3f.

The reference's parts are written by kintera::save_tensors, a library absent
here; this module writes each part with torch.save (a zip archive of the
same name -> tensor dict).  The bundle framing, the names, the index, the
reader's checks and the metadata checks are the reference's.
"""
from __future__ import annotations

import io
import os
from typing import Dict, List, Optional, Sequence

import torch

BUNDLE_MAGIC = "SNAPY_RESTART_BUNDLE_V1"
HYDRO_RESTART_VERSION = 1
HYDRO_RESTART_METADATA = "hydro_restart_metadata"
HYDRO_REFERENCE_GRID = ("hydro_ref_x1f", "hydro_ref_x2f", "hydro_ref_x3f")


class RestartError(RuntimeError):
    """A restart file that cannot be read or does not fit the block."""


def part_name(basename: str, rank: int, number: int, final: bool = False) -> str:
    return f"{basename}.block{rank}.{'final' if final else f'{number:05d}'}.part"


def restart_name(basename: str, number: int, final: bool = False) -> str:
    return f"{basename}.{'final' if final else f'{number:05d}'}.restart"


def part_rank(name: str) -> int:
    """The rank in a part name <basename>.block<rank>.<number>.part, or -1."""
    if not name.endswith(".part"):
        return -1
    stem = name[:-len(".part")]
    dot2 = stem.rfind(".")
    dot1 = stem.rfind(".", 0, dot2) if dot2 > 0 else -1
    if dot1 < 0 or not stem.startswith("block", dot1 + 1):
        return -1
    try:
        return int(stem[dot1 + 6:dot2])
    except ValueError:
        return -1


def save_part(tensors: Dict[str, torch.Tensor], path: str) -> None:
    torch.save({k: v.detach().to("cpu") for k, v in tensors.items()}, path)


def _load_part_bytes(data: bytes) -> Dict[str, torch.Tensor]:
    return torch.load(io.BytesIO(data), map_location="cpu", weights_only=True)


def make_bundle(bundle: str, parts: Sequence[str]) -> None:
    """make_restart_bundle: magic, count, '<name>\\t<bytes>' lines, an empty
    line, then the parts in index order."""
    sizes = [os.path.getsize(p) for p in parts]
    with open(bundle, "wb") as out:
        head = BUNDLE_MAGIC + "\n" + f"{len(parts)}\n"
        head += "".join(f"{os.path.basename(p)}\t{n}\n" for p, n in zip(parts, sizes))
        head += "\n"
        out.write(head.encode())
        for p in parts:
            with open(p, "rb") as f:
                while True:
                    chunk = f.read(1 << 20)
                    if not chunk:
                        break
                    out.write(chunk)


def combine(out_dir: str, basename: str, number: int, final: bool = False) -> str:
    """combine_blocks: the parts of every block into one restart file."""
    tag = "final" if final else f"{number:05d}"
    parts = sorted(
        (os.path.join(out_dir, f) for f in os.listdir(out_dir)
         if f.startswith(basename + ".block") and f.endswith(f".{tag}.part")
         and part_rank(f) >= 0),
        key=lambda p: part_rank(os.path.basename(p)))
    if not parts:
        raise RestartError(f"{out_dir}: no restart parts {basename}.block*.{tag}.part")
    outfile = os.path.join(out_dir, restart_name(basename, number, final))
    if os.path.exists(outfile):
        os.remove(outfile)
    if len(parts) == 1:
        os.replace(parts[0], outfile)
    else:
        make_bundle(outfile, parts)
        for p in parts:
            os.remove(p)
    return outfile


def load_restart(path: str, block_rank: int = 0) -> Dict[str, torch.Tensor]:
    """The restart variables of block `block_rank`, from a bundle or from a
    single part file; RestartError if the file cannot be read, the bundle is
    malformed or truncated, or it holds no part for the block."""
    try:
        f = open(path, "rb")
    except OSError:
        raise RestartError(f"{path}: failed to open restart file")
    with f:
        first = f.readline()
        if first.rstrip(b"\n").decode(errors="replace") != BUNDLE_MAGIC:
            f.seek(0)
            return _load_part_bytes(f.read())
        line = f.readline().rstrip(b"\n")
        if not line:
            raise RestartError(f"{path}: restart bundle missing entry count")
        count = int(line)
        entries = []
        for _ in range(count):
            line = f.readline()
            text = line.rstrip(b"\n").decode(errors="replace")
            if not line or "\t" not in text:
                raise RestartError(f"{path}: restart bundle index line missing tab")
            name, size = text.split("\t", 1)
            entries.append((name, int(size)))
        line = f.readline()
        if line != b"\n":
            raise RestartError(f"{path}: restart bundle header missing terminator")
        offset = f.tell()
        for name, size in entries:
            if part_rank(name) != block_rank:
                offset += size
                continue
            f.seek(offset)
            data = f.read(size)
            if len(data) != size:
                raise RestartError(f"{path}: truncated restart bundle payload")
            return _load_part_bytes(data)
    raise RestartError(f"{path}: no part for block {block_rank} in restart bundle")


def check_restart_metadata(data: Dict[str, torch.Tensor],
                           grid: Sequence[torch.Tensor],
                           perturbation_flux: bool = False) -> None:
    """The #367 checks: the hydro metadata, the stored dtype and shape, and
    the reference grid against this block's faces x1f, x2f, x3f."""
    if HYDRO_RESTART_METADATA in data:
        meta = data[HYDRO_RESTART_METADATA]
        if meta.dtype != torch.int64 or meta.dim() != 1 or meta.numel() != 2:
            raise RestartError("restart: invalid hydro restart metadata")
        if int(meta[0]) != HYDRO_RESTART_VERSION:
            raise RestartError("restart: unsupported hydro restart metadata version")
        if "hydro_ref" not in data or "hydro_u_stored" not in data:
            raise RestartError("restart: metadata requires hydro_ref and hydro_u_stored")
        stored = data["hydro_u_stored"]
        bits = {torch.float32: 32, torch.float64: 64}.get(stored.dtype, 0)
        if not bits or int(meta[1]) != bits or \
                tuple(stored.shape) != tuple(data["hydro_u"].shape):
            raise RestartError("restart: stored hydro dtype/shape disagrees with metadata")
        for key, g in zip(HYDRO_REFERENCE_GRID, grid):
            if key not in data or not torch.equal(
                    data[key], torch.as_tensor(g, dtype=torch.float64).cpu()):
                raise RestartError(f"restart: reference grid mismatch at {key}; "
                                   "remap totals and initialize a new background")
    if perturbation_flux and ("hydro_ref" not in data
                              or "hydro_ref_species" not in data):
        raise RestartError("restart: perturbation-flux requires the original "
                           "hydro_ref and hydro_ref_species")


REQUIRED = ("hydro_u", "last_time", "last_cycle", "file_number", "next_time")


def require(data: Dict[str, torch.Tensor]) -> None:
    for k in REQUIRED:
        if k not in data:
            raise RestartError(f"Restart file is missing required variable: {k}")
