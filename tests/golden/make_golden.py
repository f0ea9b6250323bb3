"""Extract the reference's known-answer values for this path into reference_kat.json.

Run in a checkout where the PICLas sources are available; the JSON it writes is committed, so the
tests never read the reference tree.

  python tests/golden/make_golden.py path-to-piclas
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_golden.py path-to-piclas")
ROOT = sys.argv[1]
RC = os.path.join(ROOT, "regressioncheck")


def csv_row(path):
    with open(path) as f:
        head = f.readline().strip().split(",")
        vals = [float(v) for v in f.readline().strip().split(",")]
    return dict(zip(head, vals))


def ini(path):
    out = {}
    with open(path) as f:
        for line in f:
            line = line.split("!")[0].strip()
            if "=" in line:
                k, v = line.split("=", 1)
                out[k.strip()] = v.strip()
    return out


def csv_list(v):
    return [t.strip() for t in v.split(",")]


def vec(v):
    return [float(t) for t in re.findall(r"[-+0-9.eE]+", v)]


def sf_plasma_ball(kat):
    """NIG_PIC_Deposition/Plasma_Ball_Shape-function-xDir: 100000 resting particles in a ball deposited on a
    4 x 4 x 1 periodic box with 1D (x) and 2D (const. in z) kernels of shape_function, shape_function_cc and
    shape_function_adaptive; PartAnalyze.csv's integrated charge is compared with the six *_ref.csv files."""
    d = os.path.join(RC, "NIG_PIC_Deposition", "Plasma_Ball_Shape-function-xDir")
    p = ini(os.path.join(d, "parameter.ini"))
    a = ini(os.path.join(d, "analyze.ini"))
    h = ini(os.path.join(d, "hopr.ini"))
    defs = {}
    with open(os.path.join(d, "hopr.ini")) as f:
        for line in f:
            m = re.match(r"\s*DEFVAR=\((\w+)\):\s*(\w+)\s*=\s*([-+0-9.eE]+)", line)
            if m:
                defs[m.group(2)] = float(m.group(3))
    li, la, ncell = defs["li"], defs["la"], int(defs["ncell"])
    assert h["nElems"].replace(" ", "") == "(/ncell,ncell,1/)"
    refs = csv_list(a["compare_data_file_reference"])
    tols = [float(t) for t in csv_list(a["compare_data_file_tolerance"])]
    kinds = csv_list(a["compare_data_file_tolerance_type"])
    dims = [int(t) for t in csv_list(p["PIC-shapefunction-dimension"])]
    dirs = [int(t) for t in csv_list(p["PIC-shapefunction-direction"])]
    case = {}
    for ref, tol, kind in zip(refs, tols, kinds):
        m = re.match(r"(\d)d_([xyz])-dir(?:-(cc|adaptive))?_ref\.csv", ref)
        dim = int(m.group(1))
        method = "shape_function" + ("_" + m.group(3) if m.group(3) else "")
        assert dim in dims and "xyz".index(m.group(2)) + 1 == dirs[dims.index(dim)]
        case[ref[:-len("_ref.csv")]] = {"dimension": dim, "direction": "xyz".index(m.group(2)) + 1,
                                        "deposition": method, "total_charge": csv_row(os.path.join(d, ref))["002-Charge"],
                                        "tolerance": tol, "tolerance_type": kind}
    kat["sf_plasma_ball"] = {
        "source": "regressioncheck/NIG_PIC_Deposition/Plasma_Ball_Shape-function-xDir/{parameter.ini,analyze.ini,hopr.ini,*_ref.csv}",
        "N": int(p["N"]), "box_lo": [-li] * 3, "box_hi": [li] * 3, "n_elems": [ncell, ncell, 1],
        "periodic_vectors": [la, la, la],
        "n_particles": int(p["Part-Species1-Init1-ParticleNumber"]),
        "charge_ic": float(p["Part-Species1-ChargeIC"]), "mpf": float(p["Part-Species1-MacroParticleFactor"]),
        "sphere_radius": float(p["Part-Species1-Init1-RadiusIC"]), "base_point": vec(p["Part-Species1-Init1-BasePointIC"]),
        "sf_radius": float(p["PIC-shapefunction-radius"]), "sf_alpha": int(p["PIC-shapefunction-alpha"]),
        "adaptive_smoothing": p["PIC-shapefunction-adaptive-smoothing"].upper().startswith("T"),
        "depo3d": True, "tracking": p["TrackingMethod"], "cases": case,
    }


def main():
    kat = {}
    d = os.path.join(RC, "NIG_PIC_Deposition", "Plasma_Ball_cell_volweight_mean")
    p = ini(os.path.join(d, "parameter.ini"))
    a = ini(os.path.join(d, "analyze.ini"))
    row = csv_row(os.path.join(d, "PartAnalyze_ref.csv"))
    kat["cvwm_plasma_ball"] = {
        "source": "regressioncheck/NIG_PIC_Deposition/Plasma_Ball_cell_volweight_mean/{parameter.ini,analyze.ini,PartAnalyze_ref.csv}",
        "N": int(p["N"]), "n_particles": int(p["Part-Species1-Init1-ParticleNumber"]),
        "charge_ic": float(p["Part-Species1-ChargeIC"]), "mpf": float(p["Part-Species1-MacroParticleFactor"]),
        "sphere_radius": float(p["Part-Species1-Init1-RadiusIC"]),
        "tracking": p["TrackingMethod"], "deposition": p["PIC-Deposition-Type"],
        "total_charge": row["002-Charge"], "tolerance_abs": float(a["compare_data_file_tolerance"]),
    }
    for case, sub in (("PIC_constant_magnetic_field_in_z_O2", "nonrel"),
                      ("PIC_constant_magnetic_field_in_z_relativistic_O2", "rel")):
        d = os.path.join(RC, "NIG_convtest_t_poisson", case)
        p = ini(os.path.join(d, "parameter.ini"))
        a = ini(os.path.join(d, "analyze.ini"))
        base = [float(v) for v in re.findall(r"[-+0-9.eE]+", p["Part-Species1-Init1-BasePointIC"])]
        kat["boris_gyration_" + sub] = {
            "source": f"regressioncheck/NIG_convtest_t_poisson/{case}/{{parameter.ini,analyze.ini}}",
            "dt": [float(v) for v in p["ManualTimeStep"].split(",")], "tend": float(p["tend"]),
            "charge": float(p["Part-Species1-ChargeIC"]), "mass": float(p["Part-Species1-MassIC"]),
            "base_point": base, "gamma": float(p.get("PIC-AnalyticInterpolationGamma", "1.0")),
            "order": float(a["analyze_convtest_t_order"]), "order_tolerance": float(a["analyze_convtest_t_tolerance"]),
        }
    sf_plasma_ball(kat)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kat.json")
    with open(out, "w") as f:
        json.dump(kat, f, indent=1, sort_keys=True)
    print(out)


if __name__ == "__main__":
    main()
