"""Extract the reference's known-answer values for this path into reference_kat.json.

Run in a checkout where the PICLas sources are available (default: /root/reference); the
JSON it writes is committed, so the tests never read the reference tree.

  python tests/golden/make_golden.py [path-to-piclas]
"""
import json
import os
import re
import sys

ROOT = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
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
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kat.json")
    with open(out, "w") as f:
        json.dump(kat, f, indent=1, sort_keys=True)
    print(out)


if __name__ == "__main__":
    main()
