"""Writes the known-answer fixtures of tests/golden from the reference's own tests.

The reference (Rust + Metal) cannot be built here, so these vectors are the
expected values its tests assert, restated as data:
  * orbit_known_answers.json -- src/mandelbulber/orbit.rs:1866-1960
    (quadratic triplex "mandelbulb power 2", classic Mandelbulb power 2, full
    Mandelbox with scale -1.5), with the closed forms the Rust tests use
    ((2.4, -3.2, -6*sqrt(5)) and dr = 2*sqrt(14); 2*sqrt(14)+1 and |z| = 14;
    (-0.6, -1.2, -1.8), dr = 7 and colour 1.2).
  * dda_contract.json -- the voxel cell-ownership / DDA / AABB cases of
    voxel_dda_contract_test, shaders/Shaders.metal:5164-5211.
Run:  python tests/golden/make_golden.py
"""
import json
import math
import os
import struct

HERE = os.path.dirname(os.path.abspath(__file__))


def next_float(x: float) -> float:
    return struct.unpack("<f", struct.pack("<I", struct.unpack("<I", struct.pack("<f", x))[0] + 1))[0]


def main():
    orbit = {
        "source": "src/mandelbulber/orbit.rs:1866-1960",
        "cases": [
            {"name": "mandelbulb_power2_triplex", "formula": "mandelbulb_power2", "point": [1.0, 2.0, 3.0, 0.0],
             "expect": {"z": [2.4, -3.2, -6.0 * math.sqrt(5.0), 0.0], "derivative": 2.0 * math.sqrt(14.0)},
             "tolerance": 1e-12, "source": "src/mandelbulber/orbit.rs:1866-1874"},
            {"name": "classic_mandelbulb_power2", "formula": "mandelbulb", "power": 2.0, "point": [1.0, 2.0, 3.0, 0.0],
             "expect": {"derivative": 2.0 * math.sqrt(14.0) + 1.0, "length": 14.0}, "tolerance": 1e-12},
            {"name": "full_mandelbox_unrotated", "formula": "mandelbox", "scale": -1.5, "folding_limit": 1.0,
             "folding_value": 2.0, "fixed_radius": 1.0, "minimum_radius": 0.5, "point": [0.1, 0.2, 0.3, 0.0],
             "expect": {"z": [-0.6, -1.2, -1.8, 0.0], "derivative": 7.0, "color": 1.2}, "tolerance": 1e-12},
        ],
    }
    with open(os.path.join(HERE, "orbit_known_answers.json"), "w") as f:
        json.dump(orbit, f, indent=1)
    dda = {
        "source": "shaders/Shaders.metal:5164-5211",
        "bounds_min": [0.0, 0.0, 0.0], "bounds_max": [4.0, 4.0, 4.0], "cell_size": [1.0, 1.0, 1.0], "resolution": 4,
        "cell_coordinate": [
            {"point": [1.0, 2.0, 3.0], "direction": [1.0, 1.0, 1.0], "ok": True, "cell": [1, 2, 3]},
            {"point": [1.0, 2.0, 3.0], "direction": [-1.0, -1.0, -1.0], "ok": True, "cell": [0, 1, 2]},
            {"point": [4.0, 4.0, 4.0], "direction": [-1.0, -1.0, -1.0], "ok": True, "cell": [3, 3, 3]},
            {"point": [4.0, 4.0, 4.0], "direction": [1.0, 1.0, 1.0], "ok": False},
            {"point": [4.0, 4.0, 4.0], "direction": [0.0, 0.0, 0.0], "ok": True, "cell": [3, 3, 3]},
        ],
        "advance": [
            {"cell": [0, 0, 0], "step": [1, 1, 1], "next_t": [1.0, 1.0, 2.0], "delta_t": [1.0, 1.0, 1.0], "entry_t": 0.0,
             "expect": [{"cell": [1, 1, 0], "next_t": [2.0, 2.0, 2.0], "entry_t": 1.0, "normal": [-1.0, 0.0, 0.0]},
                        {"cell": [2, 2, 1], "next_t": [3.0, 3.0, 3.0], "entry_t": 2.0}]},
            {"cell": [0, 0, 0], "step": [1, 1, 1], "next_t": [1.0, 2.0, 3.0], "delta_t": [1.0, 1.0, 1.0], "entry_t": 1.0,
             "expect": [{"cell": [1, 0, 0], "entry_t": next_float(1.0)}]},
        ],
        "aabb": [
            {"origin": [-1.0, 2.0, 2.0], "direction": [1e-9, 0.0, 0.0], "hit": True, "near_positive": True},
            {"origin": [-1.0, 5.0, 2.0], "direction": [1.0, 0.0, 0.0], "hit": False},
        ],
    }
    with open(os.path.join(HERE, "dda_contract.json"), "w") as f:
        json.dump(dda, f, indent=1)


if __name__ == "__main__":
    main()
