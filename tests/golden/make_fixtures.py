"""Extracts the golden vectors this project pins its oracle to from kiyosi's benchmark
calibration records (benchmarks/quantlib/calibration/*.json, produced by the kiyosi
0.19.0 build) and reference values (benchmarks/quantlib/references/*.json).

Run in a checkout that has the reference mounted:
    python tests/golden/make_fixtures.py /path/to/kiyosi
Writes european_calibration.json, barrier_calibration.json, american_calibration.json,
known_answers.json and local_volatility_structured.json (from the reference's QuantLib
local-volatility fixture, python/tests/quantlib_reference/) here.
"""
import ast
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _parse(v):
    return ast.literal_eval(v) if isinstance(v, str) else v


def main(root):
    cal = os.path.join(root, "benchmarks", "quantlib", "calibration")
    ref = os.path.join(root, "benchmarks", "quantlib", "references")
    mc = json.load(open(os.path.join(cal, "monte_carlo.json")))
    rows = []
    for e in mc["experiments"]:
        if e["backend"] != "kiyosi" or e["id"] not in ("mc-european-call", "mc-european-put"):
            continue
        ens = _parse(e["seed_ensemble"])
        for s in ens["samples"]:
            p = s["profile"]
            rows.append({"id": e["id"], "seed": s["seed"], "path_count": p["path_count"],
                         "price": s["price"]})
        prof = _parse(e["profile"])
        timing = _parse(e["timing_seed_accuracy"])
        rows.append({"id": e["id"], "seed": prof["seed"], "path_count": prof["path_count"],
                     "price": timing["price"]})
    inputs = {"spot": 100.0, "strike": 100.0, "rate": 0.05, "dividend": 0.02, "volatility": 0.2,
              "expiry_years": 1.0, "valuation": "2025-01-01", "expiry": "2026-01-01"}
    json.dump({"source": "benchmarks/quantlib/calibration/monte_carlo.json (kiyosi "
                         + mc["libraries"]["kiyosi"]["version"] + ")",
               "inputs": inputs, "samples": rows},
              open(os.path.join(HERE, "european_calibration.json"), "w"), indent=1)
    # Continuously monitored barriers of the same calibration (one terminal draw).
    cases = {c["id"]: c for c in json.load(open(os.path.join(root, "benchmarks", "quantlib", "cases",
                                                             "monte_carlo.json")))["cases"]}
    brows = []
    for e in mc["experiments"]:
        if e["backend"] != "kiyosi" or e["id"] not in ("mc-barrier-down-out-call", "mc-barrier-up-in-put"):
            continue
        ens = _parse(e["seed_ensemble"])
        for s in ens["samples"]:
            brows.append({"id": e["id"], "seed": s["seed"], "path_count": s["profile"]["path_count"],
                          "price": s["price"]})
        prof = _parse(e["profile"])
        brows.append({"id": e["id"], "seed": prof["seed"], "path_count": prof["path_count"],
                      "price": _parse(e["timing_seed_accuracy"])["price"]})
    binputs = {k: cases[k]["inputs"] for k in ("mc-barrier-down-out-call", "mc-barrier-up-in-put")}
    json.dump({"source": "benchmarks/quantlib/calibration/monte_carlo.json (kiyosi "
                         + mc["libraries"]["kiyosi"]["version"] + ")",
               "inputs": binputs, "samples": brows},
              open(os.path.join(HERE, "barrier_calibration.json"), "w"), indent=1)
    am = json.load(open(os.path.join(cal, "american_monte_carlo.json")))
    arows = []
    for e in am["experiments"]:
        if e["backend"] != "kiyosi":
            continue
        ens = _parse(e["seed_ensemble"])
        for s in ens["samples"]:
            p = s["profile"]
            arows.append({"seed": s["seed"], "path_count": p["path_count"],
                          "step_count": p["step_count"], "antithetic": p["antithetic"],
                          "sampling": p["sampling"], "price": s["price"]})
    json.dump({"source": "benchmarks/quantlib/calibration/american_monte_carlo.json (kiyosi "
                         + am["libraries"]["kiyosi"]["version"] + ")",
               "inputs": dict(inputs, option="put"), "samples": arows},
              open(os.path.join(HERE, "american_calibration.json"), "w"), indent=1)
    known = {}
    for name in ("monte_carlo.json", "american_monte_carlo.json", "heston.json"):
        path = os.path.join(ref, name)
        if not os.path.exists(path):
            continue
        data = json.load(open(path))
        for r in data["cases"]:
            prov = _parse(r.get("provenance", "{}"))
            known[r["id"]] = {"value": float(r["value"]),
                              "uncertainty": float(r["uncertainty"]),
                              "inputs": prov.get("inputs") if isinstance(prov, dict) else None}
    json.dump({"source": "benchmarks/quantlib/references/*.json", "values": known},
              open(os.path.join(HERE, "known_answers.json"), "w"), indent=1)
    # QuantLib local-volatility paths of the structured notes (the reference's Python test
    # fixture; prices with antithetic-pair standard errors and the time-refinement bias).
    lv = json.load(open(os.path.join(root, "python", "tests", "quantlib_reference",
                                     "local_volatility_structured.json")))
    keep = {k: lv["reference"][k] for k in ("quantlib_version", "pairs", "substeps_per_day",
                                             "time_steps", "seed", "spot", "results")}
    json.dump({"source": "python/tests/quantlib_reference/local_volatility_structured.json "
                         "(generator local_volatility_paths.py)",
               "reference": keep, "time_refinement": lv["time_refinement"][-1]},
              open(os.path.join(HERE, "local_volatility_structured.json"), "w"), indent=1)
    print(len(rows), "European rows,", len(brows), "barrier rows,", len(arows), "American rows,",
          len(known), "known answers,", len(keep["results"]), "local-volatility notes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <path of the kiyosi checkout>")
    main(sys.argv[1])
