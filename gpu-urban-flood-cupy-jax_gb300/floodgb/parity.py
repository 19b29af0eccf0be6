"""Snapshot-by-snapshot parity figures between a reference run and a candidate
run of the same scenario (NumPy, host side).

This restates the per-snapshot arithmetic of the reference's
``validate_v1_parity_run`` (hybrid_flood/operational/parity_validation.py:
43-253): over the valid cells (active, not building), the depth RMSE, the
wet-cell RMSE, the 99th-percentile absolute error and the flood-extent CSI
at 0.05 m (:99-124), the surface volume of all cells against the cell areas
and its relative error (:35-36, 115-116), the final node-volume / link-flow
errors (:128-153) and the summary maxima (:168-177).  It works on arrays, so
it compares two runs held in memory (a candidate and a reference run of the
same scenario) as well as two written output directories.

The gates are two sets: the reference's own V1-parity gates (:179-192, RMSE
<= 0.05 m, CSI >= 0.95, volume <= 2 %) and the tighter drop-in gates this
library is held to (RMSE <= 1e-3 m, CSI >= 0.995, volume <= 0.05 %).

The reference scores a snapshot where neither run has a wet cell (an early
snapshot of a dry start) as CSI 0 (intersection / max(union, 1)); the rows
keep that figure, and the drop-in CSI gate reads ``extent_agreement_csi``,
which counts two empty extents as agreeing (1.0) and equals the reference's
CSI whenever anything is wet.
"""

from __future__ import annotations

import numpy as np

DEPTH_THRESHOLD_M = 0.05

#: drop-in gates: (summary key, bound, "max" | "min")
DROP_IN_GATES = {
    "depth_rmse_le_1mm": ("maximum_snapshot_valid_depth_rmse_m", 1.0e-3, "max"),
    "csi_ge_0_995": ("minimum_snapshot_extent_agreement_csi", 0.995, "min"),
    "volume_error_le_0_05pct": ("maximum_snapshot_surface_volume_error_fraction", 5.0e-4, "max"),
}


def _relative(candidate: float, reference: float) -> float:
    # parity_validation.py:35-36
    return (candidate - reference) / max(abs(reference), 1.0)


def snapshot_row(ref_depth, cand_depth, valid, area, threshold_m: float = DEPTH_THRESHOLD_M) -> dict:
    """Figures of one aligned snapshot (parity_validation.py:99-124)."""

    ref_depth = np.asarray(ref_depth, np.float32)
    cand_depth = np.asarray(cand_depth, np.float32)
    r = ref_depth[valid].astype(np.float64)
    c = cand_depth[valid].astype(np.float64)
    diff = c - r
    ref_wet = r >= threshold_m
    cand_wet = c >= threshold_m
    union = ref_wet | cand_wet
    inter = ref_wet & cand_wet
    vr = float(np.sum(ref_depth.astype(np.float64) * area))
    vc = float(np.sum(cand_depth.astype(np.float64) * area))
    return {
        "valid_depth_rmse_m": float(np.sqrt(np.mean(diff ** 2))) if diff.size else 0.0,
        "reference_wet_depth_rmse_m": float(np.sqrt(np.mean(diff[ref_wet] ** 2))) if ref_wet.any() else 0.0,
        "depth_absolute_error_p99_m": float(np.percentile(np.abs(diff), 99)) if diff.size else 0.0,
        "max_absolute_error_m": float(np.max(np.abs(diff))) if diff.size else 0.0,
        "flood_extent_csi": float(inter.sum() / max(int(union.sum()), 1)),
        "extent_agreement_csi": float(inter.sum() / union.sum()) if union.any() else 1.0,
        "reference_wet_triangle_count": int(ref_wet.sum()),
        "candidate_wet_triangle_count": int(cand_wet.sum()),
        "reference_surface_volume_m3": vr,
        "candidate_surface_volume_m3": vc,
        "surface_volume_error_fraction": _relative(vc, vr),
        "reference_max_depth_m": float(np.max(r)) if r.size else 0.0,
        "candidate_max_depth_m": float(np.max(c)) if c.size else 0.0,
    }


def compare_runs(ref_times, ref_depth, cand_times, cand_depth, valid, area, *, threshold_m: float = DEPTH_THRESHOLD_M,
                 ref_node_volume=None, cand_node_volume=None, ref_link_flow=None, cand_link_flow=None,
                 ref_ledger: dict | None = None, cand_ledger: dict | None = None) -> dict:
    """Per-snapshot rows, drainage-state errors, ledger comparison, summary and
    both gate sets for two runs with aligned snapshots (same count)."""

    ref_times = np.asarray(ref_times, np.float64)
    cand_times = np.asarray(cand_times, np.float64)
    ref_depth = np.asarray(ref_depth)
    cand_depth = np.asarray(cand_depth)
    if ref_depth.shape != cand_depth.shape or ref_times.shape != cand_times.shape:
        raise ValueError(f"Parity shape mismatch: reference {ref_depth.shape}/{ref_times.shape}, "
                         f"candidate {cand_depth.shape}/{cand_times.shape}.")
    valid = np.asarray(valid, bool)
    area = np.asarray(area, np.float64)
    if valid.shape != ref_depth.shape[1:] or area.shape != valid.shape:
        raise ValueError("Domain mask / cell areas do not match the snapshots.")
    rows = []
    for k in range(ref_depth.shape[0]):
        row = {"snapshot_index": k, "reference_time_s": float(ref_times[k]), "candidate_time_s": float(cand_times[k]),
               "time_delta_s": float(cand_times[k] - ref_times[k])}
        row.update(snapshot_row(ref_depth[k], cand_depth[k], valid, area, threshold_m))
        rows.append(row)
    drainage = {}
    if ref_node_volume is not None and cand_node_volume is not None and np.size(ref_node_volume):
        d = np.asarray(cand_node_volume, np.float64) - np.asarray(ref_node_volume, np.float64)
        drainage.update({"final_node_volume_rmse_m3": float(np.sqrt(np.mean(d ** 2))),
                         "final_node_volume_mae_m3": float(np.mean(np.abs(d))),
                         "final_node_volume_max_absolute_error_m3": float(np.max(np.abs(d)))})
    if ref_link_flow is not None and cand_link_flow is not None and np.size(ref_link_flow):
        d = np.asarray(cand_link_flow, np.float64) - np.asarray(ref_link_flow, np.float64)
        drainage.update({"final_link_flow_rmse_m3ps": float(np.sqrt(np.mean(d ** 2))),
                         "final_link_flow_mae_m3ps": float(np.mean(np.abs(d))),
                         "final_link_flow_max_absolute_error_m3ps": float(np.max(np.abs(d)))})
    ledger = {}
    if ref_ledger and cand_ledger:
        for name, rv in ref_ledger.items():
            if name in cand_ledger:
                ledger[name] = {"reference": float(rv), "candidate": float(cand_ledger[name]),
                                "relative_error_fraction": _relative(float(cand_ledger[name]), float(rv))}
    finite = bool(np.isfinite(cand_depth).all() and (cand_depth.size == 0 or np.min(cand_depth) >= -1.0e-7))
    summary = {
        "snapshots": len(rows),
        "maximum_snapshot_time_delta_s": max((abs(r["time_delta_s"]) for r in rows), default=0.0),
        "maximum_snapshot_valid_depth_rmse_m": max((r["valid_depth_rmse_m"] for r in rows), default=0.0),
        "minimum_snapshot_flood_extent_csi": min((r["flood_extent_csi"] for r in rows), default=1.0),
        "minimum_snapshot_extent_agreement_csi": min((r["extent_agreement_csi"] for r in rows), default=1.0),
        "maximum_snapshot_surface_volume_error_fraction": max(
            (abs(r["surface_volume_error_fraction"]) for r in rows), default=0.0),
        "maximum_snapshot_max_absolute_error_m": max((r["max_absolute_error_m"] for r in rows), default=0.0),
        "maximum_source_sink_ledger_error_fraction": max(
            (abs(v["relative_error_fraction"]) for v in ledger.values()), default=0.0),
    }
    reference_gates = {
        "finite_non_negative_depth": finite,
        "snapshot_alignment_le_1s": summary["maximum_snapshot_time_delta_s"] <= 1.0,
        "all_snapshot_depth_rmse_le_0_05m": summary["maximum_snapshot_valid_depth_rmse_m"] <= 0.05,
        "all_snapshot_csi_ge_0_95": summary["minimum_snapshot_flood_extent_csi"] >= 0.95,
        "all_snapshot_volume_error_le_2pct": summary["maximum_snapshot_surface_volume_error_fraction"] <= 0.02,
    }
    drop_in = {}
    for name, (key, bound, kind) in DROP_IN_GATES.items():
        drop_in[name] = summary[key] <= bound if kind == "max" else summary[key] >= bound
    drop_in["finite_non_negative_depth"] = finite
    # passed: every drop-in gate and every reference gate but its CSI one, which
    # the tighter drop-in CSI gate replaces (it differs only on all-dry snapshots)
    passed = all(drop_in.values()) and all(v for k, v in reference_gates.items() if k != "all_snapshot_csi_ge_0_95")
    return {"threshold_m": threshold_m, "snapshots": rows, "drainage_state": drainage, "ledger_comparison": ledger,
            "summary": summary, "reference_gates": reference_gates, "drop_in_gates": drop_in, "passed": passed}
