"""Run files: the reference's npz + JSON manifest, version 1.

Format of utils/data_io.py:27-75 (kept so the reference's ``load_runs`` and
``*Analysis.from_file`` read these files, and ``load_runs`` here reads
theirs): one zip archive with a ``.npy`` member ``L{L}_{name}`` per sample
channel of each run and a ``manifest`` member holding a 0-d unicode array of
the JSON text ``{"version": 1, "runs": {"<L>": {"metadata": ...,
"sample_names": [...]}}}``.

``save_runs`` writes the members itself with zlib level 1 (level 6 is what
``numpy.savez_compressed`` uses): the archive format and contents are the
same, deflate at level 1 is several times faster on float64 samples.  It
writes to a temporary file next to the target and renames it, so a failed
save leaves no partial file.
"""

import io
import json
import os
import tempfile
import zipfile
from pathlib import Path

import numpy as np

FORMAT_VERSION = 1


def json_ready(value):
    """NumPy metadata -> JSON values (utils/data_io.py:6-24)."""
    if isinstance(value, np.ndarray):
        return value.tolist()
    if isinstance(value, np.generic):
        return value.item()
    if isinstance(value, dict):
        return {str(k): json_ready(v) for k, v in value.items()}
    if isinstance(value, (list, tuple)):
        return [json_ready(v) for v in value]
    return value


def _npy_bytes(array):
    buf = io.BytesIO()
    np.lib.format.write_array(buf, np.asanyarray(array), allow_pickle=False)
    return buf.getvalue()


def save_runs(path, runs, compresslevel=1):
    """Write ``{L: {"samples": {name: array}, "metadata": dict}}`` to ``path``."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    manifest = {"version": FORMAT_VERSION, "runs": {}}
    members = []
    for L, run in runs.items():
        samples = run["samples"]
        manifest["runs"][str(L)] = {"metadata": json_ready(run["metadata"]), "sample_names": list(samples)}
        for name, values in samples.items():
            members.append((f"L{L}_{name}.npy", np.asarray(values)))
    members.append(("manifest.npy", np.array(json.dumps(manifest))))

    fd, tmp = tempfile.mkstemp(prefix=path.name + ".", suffix=".tmp", dir=path.parent)
    try:
        with os.fdopen(fd, "wb") as f, zipfile.ZipFile(f, "w", compression=zipfile.ZIP_DEFLATED,
                                                        compresslevel=compresslevel, allowZip64=True) as zf:
            for name, array in members:
                zf.writestr(name, _npy_bytes(array))
        os.replace(tmp, path)
    except BaseException:
        try:
            os.unlink(tmp)
        except OSError:
            pass
        raise


def load_runs(path):
    """Read a version-1 run file: ``{L: {"samples": ..., "metadata": ...}}``."""
    runs = {}
    with np.load(path, allow_pickle=False) as f:
        manifest = json.loads(f["manifest"].item())
        if manifest["version"] != FORMAT_VERSION:
            raise ValueError("Unsupported data format version")
        for L_str, info in manifest["runs"].items():
            L = int(L_str)
            runs[L] = {"samples": {name: f[f"L{L}_{name}"].copy() for name in info["sample_names"]},
                       "metadata": info["metadata"]}
    return runs


def runs_by_size(runs):
    """``LadderBatch.simulate`` output (a list, one run per ladder) as the
    ``{L: run}`` mapping a run file holds; a size may appear once."""
    out = {}
    for run in runs:
        L = int(run["metadata"]["L"])
        if L in out:
            raise ValueError(f"L={L} appears in more than one ladder; save them to separate files")
        out[L] = run
    return out
