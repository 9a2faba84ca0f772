"""File formats and drivers for the oracle (test infrastructure only -- never on the product path).

* model file (``DNLM``): written by :func:`write_model`, read by ``ref_harness`` (oracle/ref_harness.C)
* state file (``DNST``): nodal + integration-point state injected by ``ref_harness forces``
* record file: the harness' output, a sequence of named float64 arrays (:func:`read_records`)

:func:`run_reference` runs the compiled reference (``oracle/_ref/ref_harness``), which exists only
where the reference sources could be compiled (this container, not the GPU machine).
"""

from __future__ import annotations

import os
import struct
import subprocess
import tempfile
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")

MODEL_MAGIC = 0x4D4C4E44  # "DNLM"
EXT_MAGIC = 0x584C4E44  # "DNLX": optional block after the solver settings
STATE_MAGIC = 0x54534E44  # "DNST"
MIXED = 9  # model file etype: the elements' own types follow


def write_model(path: str, m) -> None:
    """Serialise a :class:`redynela_gb300.meshes.Model` for the harness."""
    groups = m.element_groups() if hasattr(m, "element_groups") else [(m.etype, m.conn)]
    with open(path, "wb") as f:
        if len(groups) == 1:
            f.write(struct.pack("<4q", MODEL_MAGIC, m.etype, m.N, m.E))
            f.write(np.ascontiguousarray(m.coords, dtype="<f8").tobytes())
            f.write(np.ascontiguousarray(m.conn, dtype="<i8").tobytes())
        else:
            # etype 9: the type of each element, then every element's nodes
            E = sum(c.shape[0] for _, c in groups)
            f.write(struct.pack("<4q", MODEL_MAGIC, MIXED, m.N, E))
            f.write(np.ascontiguousarray(m.coords, dtype="<f8").tobytes())
            types = np.concatenate([np.full(c.shape[0], t, dtype="<i8") for t, c in groups])
            f.write(types.tobytes())
            for _, c in groups:
                f.write(np.ascontiguousarray(c, dtype="<i8").tobytes())
        f.write(struct.pack("<6d", m.young, m.poisson, m.density, m.A, m.B, m.n))
        f.write(struct.pack("<3d", *m.v0))
        f.write(struct.pack("<q", len(m.bcs)))
        for g in m.bcs:
            f.write(struct.pack("<q3dq", g.kind, *g.val, len(g.nodes)))
            f.write(np.ascontiguousarray(g.nodes, dtype="<i8").tobytes())
        f.write(struct.pack("<6d", m.tend, m.rho_b, m.safety, float(m.freq), float(m.method),
                            float(m.nsaves)))
        if getattr(m, "extended", False):
            # materials / laws, element materials, per-node initial velocities
            laws = m.material_laws()
            f.write(struct.pack("<2q", EXT_MAGIC, len(laws)))
            for ml in laws:
                prm = list(ml.params) + [0.0] * (8 - len(ml.params))
                tx = np.zeros(0) if ml.table_x is None else np.asarray(ml.table_x, dtype="<f8")
                ty = np.zeros(0) if ml.table_y is None else np.asarray(ml.table_y, dtype="<f8")
                f.write(struct.pack("<3dq8dq", ml.young, ml.poisson, ml.density, ml.law, *prm, tx.size))
                f.write(tx.tobytes())
                f.write(ty.tobytes())
            em = m.elem_material
            f.write(struct.pack("<q", 0 if em is None else 1))
            if em is not None:
                f.write(np.ascontiguousarray(em, dtype="<i8").tobytes())
            iv = m.initial_velocity
            f.write(struct.pack("<q", 0 if iv is None else 1))
            if iv is not None:
                f.write(np.ascontiguousarray(iv, dtype="<f8").tobytes())


def write_state(path: str, coords, du, v, a, disp, S, Eps, EpsPlas, p, evp, dt) -> None:
    """Nodal arrays are (N, 3); tensors are (E, nip, 3, 3) or, for any mix of element types,
    (nIP, 3, 3) in element order; p, evp are (E, nip) or (nIP,)."""
    N = coords.shape[0]
    node = np.concatenate([coords, du, v, a, disp], axis=1).reshape(N, 15)
    ip = np.concatenate([S.reshape(-1, 9), Eps.reshape(-1, 9), EpsPlas.reshape(-1, 9),
                         p.reshape(-1, 1), evp.reshape(-1, 1)], axis=1)
    with open(path, "wb") as f:
        f.write(struct.pack("<q", STATE_MAGIC))
        f.write(np.ascontiguousarray(node, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(ip, dtype="<f8").tobytes())
        f.write(struct.pack("<d", dt))


def read_records(path: str) -> Dict[str, np.ndarray]:
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        (ln,) = struct.unpack_from("<q", data, pos)
        pos += 8
        name = data[pos:pos + ln].decode()
        pos += ln
        (cnt,) = struct.unpack_from("<q", data, pos)
        pos += 8
        out[name] = np.frombuffer(data, dtype="<f8", count=cnt, offset=pos).copy()
        pos += 8 * cnt
    return out


def reference_tables() -> Dict[str, np.ndarray]:
    """Shape-function tables of the reference elements (ref_harness tables)."""
    with tempfile.TemporaryDirectory(prefix="dnlref_") as tmp:
        out = os.path.join(tmp, "tables.rec")
        subprocess.run([REF_HARNESS, "tables", out], cwd=tmp, check=True, capture_output=True)
        return read_records(out)


def reference_available() -> bool:
    return os.path.exists(REF_HARNESS)


def run_reference(cmd: str, model, *extra, state: Optional[dict] = None, threads: int = 1,
                  timeout: float = 3600.0, strategy: Optional[int] = None) -> Dict[str, np.ndarray]:
    """Run ``ref_harness <cmd>`` on ``model`` in a scratch directory and return its records.
    ``strategy``: the reference's Domain::computeInternalForces parallelisation (0-7, the
    ``computeInternalForces`` environment variable it reads, Domain.C:148-152); default 0."""
    if not reference_available():
        raise RuntimeError("compiled reference not found: run `make -C oracle ref` first")
    with tempfile.TemporaryDirectory(prefix="dnlref_") as tmp:
        mpath = os.path.join(tmp, "model.dnlm")
        out = os.path.join(tmp, "out.rec")
        write_model(mpath, model)
        args = [REF_HARNESS, cmd, mpath]
        if cmd == "forces":
            spath = os.path.join(tmp, "state.dnst")
            write_state(spath, **state)
            args += [spath, out]
        else:
            args += [out] + [str(x) for x in extra]
        env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_DYNAMIC="FALSE")
        env.pop("computeInternalForces", None)
        if strategy is not None:
            env["computeInternalForces"] = str(int(strategy))
        r = subprocess.run(args, cwd=tmp, env=env, capture_output=True, text=True,
                           timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"ref_harness {cmd} failed ({r.returncode}):\n{r.stderr[-2000:]}")
        rec = read_records(out)
        plots = [f for f in os.listdir(tmp) if f.endswith(".plot")]
        plot = os.path.join(tmp, plots[0]) if plots else ""
        if plot and os.path.exists(plot):
            rows = [ln.split() for ln in open(plot) if ln.strip() and not ln.startswith("#")]
            rec["plot"] = np.array(rows, dtype=np.float64).reshape(-1, 4) if rows else np.zeros((0, 4))
        return rec
