"""Per-step error of the mixed-precision loop against the FP64 loop on the same inputs.

Both variants run side by side through the C-ABI (fused ``pic_step`` one step at a time).  After
each step the report takes, for each output, the infinity norm of the difference relative to the
infinity norm of the FP64 value:

* ``rho``  -- ``PartSource(4,:)`` deposited at the start of the step (``Deposition``);
* ``E``    -- ``FieldAtParticle(1:3,:)`` at the positions after the step (``InterpolateFieldToParticle``
  of the state the next step starts from);
* ``x``    -- positions, as the minimum-image distance in metres (the box is periodic);
* ``v``    -- velocities;
* ``elem_mismatch`` -- particles whose element differs (must stay 0: element ids are exact).
"""
from __future__ import annotations

import numpy as np

from . import ParticleLoop, capi


def _rel_inf(a: np.ndarray, b: np.ndarray) -> float:
    den = float(np.max(np.abs(b))) if b.size else 0.0
    return float(np.max(np.abs(a - b)) / den) if den > 0 else float(np.max(np.abs(a - b), initial=0.0))


def mixed_vs_fp64_per_step(w, nsteps: int, sort_interval: int = 0) -> list[dict]:
    """Run ``w`` in FP64 and in the mixed variant for ``nsteps`` steps; one error row per step."""
    loops = {}
    for prec in (capi.PIC_PREC_FP64, capi.PIC_PREC_MIXED):
        loop = ParticleLoop(w.config(precision=prec, sort_interval=sort_interval), w.mesh)
        loop.set_field(w.e_dof)
        loop.upload_particles(w.part_state, w.elem, w.part_species)
        loops[prec] = loop
    box = np.asarray(w.mesh.hi, dtype=np.float64) - np.asarray(w.mesh.lo, dtype=np.float64)
    rows = []
    try:
        for k in range(nsteps):
            res = {}
            for prec, loop in loops.items():
                PS = np.zeros(w.mesh.dof_shape(4))
                loop.time_step(w.dt, 1, PS)
                loop.interpolate_field_to_particle()
                F = loop.field_at_particles()
                g = loop.download_particles()
                res[prec] = (PS, F, g)
            PS64, F64, g64 = res[capi.PIC_PREC_FP64]
            PS32, F32, g32 = res[capi.PIC_PREC_MIXED]
            dx = g32["part_state"][:, :3] - g64["part_state"][:, :3]
            dx -= box * np.round(dx / box)
            rows.append({
                "step": k + 1,
                "rho": _rel_inf(PS32[..., 3], PS64[..., 3]),
                "E": _rel_inf(F32[:, :3], F64[:, :3]),
                "x_m": float(np.max(np.abs(dx), initial=0.0)),
                "v": _rel_inf(g32["part_state"][:, 3:], g64["part_state"][:, 3:]),
                "elem_mismatch": int((g32["elem"] != g64["elem"]).sum()),
            })
    finally:
        for loop in loops.values():
            loop.close()
    return rows


def summarize(rows: list[dict]) -> dict:
    """Maximum over steps of each error, the last step's row, and a per-10-step excerpt."""
    keys = ("rho", "E", "x_m", "v", "elem_mismatch")
    return {"steps": len(rows),
            "max": {k: max(r[k] for r in rows) for k in keys} if rows else {},
            "last": rows[-1] if rows else {},
            "every_10": [r for r in rows if r["step"] % 10 == 0]}
