"""Fluid / simulation property files and the derived parameter block.

Mirrors `sph_simulation::load_settings` (libclsph/sph_simulation.cpp:405-505):
the two JSON files (fluid_properties/*.json, simulation_properties/*.json,
whose objects end with `};`), the restitution range check, and the derived
h, time_delta, max_velocity and the five smoothing-kernel constants with the
reference's float/double mixing:

  total_mass     = float(N) * m                          (float)
  initial_volume = total_mass / rho0                     (float)
  h              = cbrtf( float( 3f*(k*(V/N)) / (4f*M_PI) ) )   (double divide)
  time_delta     = 1f / fps
  max_velocity   = 0.8f * h / time_delta
  poly_6         = float( 315 / (64 * M_PI * pow(h, 9)) )    (double)
  poly_6_gradient = poly_6_laplacian = float( -945 / (32 * M_PI * pow(h, 9)) )
  spiky          = float( -45 / (M_PI * pow(h, 6)) ),  viscosity = -spiky
"""

from __future__ import annotations

import ctypes
import ctypes.util
import json
import math
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from .layout import PARAMS, TERMS

f32 = np.float32

_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.cbrtf.restype = ctypes.c_float
_libm.cbrtf.argtypes = [ctypes.c_float]


def cbrtf(x) -> np.float32:
    """C's cbrtf (the reference calls it; numpy's float32 cbrt can differ by an ulp)."""
    return f32(_libm.cbrtf(float(f32(x))))

FLUID_KEYS = ["fluid_density", "dynamic_viscosity", "restitution", "k",
              "surface_tension_threshold", "surface_tension", "particles_inside_influence_radius"]
SIM_KEYS = ["particles_count", "particle_mass", "simulation_time", "target_fps",
            "simulation_scale", "constant_acceleration", "write_all_frames", "serialize"]


def read_property_file(path: str | Path) -> dict:
    """First JSON object of the file; trailing text such as `;` is ignored, as
    picojson's stream parse does."""
    text = Path(path).read_text()
    obj, _ = json.JSONDecoder().raw_decode(text.lstrip())
    if not isinstance(obj, dict):
        raise ValueError(f"{path}: top-level JSON value is not an object")
    return obj


@dataclass
class Settings:
    params: np.void          # PARAMS record
    terms: np.void           # TERMS record
    initial_volume: float
    write_intermediate_frames: bool
    serialize: bool


def derive(params: np.void, influence_count: int) -> tuple[np.void, np.void, float]:
    """Derived fields of sph_simulation.cpp:490-505 (see module docstring)."""
    p = np.zeros(1, dtype=PARAMS)  # zeroed padding: the record is compared and passed as bytes
    p[0] = params
    n = int(p["particles_count"][0])
    m = f32(p["particle_mass"][0])
    total_mass = f32(f32(n) * m)
    volume = f32(total_mass / f32(p["fluid_density"][0]))
    q = float(f32(3.0) * f32(f32(influence_count) * f32(volume / f32(n)))) / (4.0 * math.pi)
    h = cbrtf(q)
    td = f32(f32(1.0) / f32(p["target_fps"][0]))
    p["total_mass"] = total_mass
    p["h"] = h
    p["time_delta"] = td
    p["max_velocity"] = f32(f32(f32(0.8) * h) / td)
    hd = float(h)
    t = np.zeros(1, dtype=TERMS)
    t["poly_6"] = f32(315.0 / (64.0 * math.pi * math.pow(hd, 9.0)))
    t["poly_6_gradient"] = f32(-945.0 / (32.0 * math.pi * math.pow(hd, 9.0)))
    t["poly_6_laplacian"] = f32(-945.0 / (32.0 * math.pi * math.pow(hd, 9.0)))
    t["spiky"] = f32(-45.0 / (math.pi * math.pow(hd, 6.0)))
    t["viscosity"] = f32(45.0 / (math.pi * math.pow(hd, 6.0)))
    return p[0], t[0], float(volume)


def settings_from_dicts(fluid: dict, sim: dict) -> Settings:
    missing = [k for k in FLUID_KEYS if k not in fluid] + [k for k in SIM_KEYS if k not in sim]
    if missing:
        raise KeyError(f"missing property keys: {missing}")
    p = np.zeros(1, dtype=PARAMS)
    p["fluid_density"] = float(fluid["fluid_density"])
    p["dynamic_viscosity"] = float(fluid["dynamic_viscosity"])
    restitution = f32(float(fluid["restitution"]))
    if restitution < 0 or restitution > 1:  # sph_simulation.cpp:423-425
        raise ValueError("Restitution has an invalid value!")
    p["restitution"] = restitution
    p["K"] = float(fluid["k"])
    p["surface_tension_threshold"] = float(fluid["surface_tension_threshold"])
    p["surface_tension"] = float(fluid["surface_tension"])
    influence = int(float(fluid["particles_inside_influence_radius"]))
    p["particles_count"] = int(float(sim["particles_count"]))
    p["particle_mass"] = float(sim["particle_mass"])
    p["simulation_time"] = float(sim["simulation_time"])
    p["target_fps"] = float(sim["target_fps"])
    p["simulation_scale"] = float(sim["simulation_scale"])
    acc = sim["constant_acceleration"]
    p["constant_acceleration"][0, :3] = [float(acc["x"]), float(acc["y"]), float(acc["z"])]
    params, terms, volume = derive(p[0], influence)
    return Settings(params, terms, volume, bool(sim["write_all_frames"]), bool(sim["serialize"]))


def load_settings(fluid_file: str | Path, params_file: str | Path) -> Settings:
    """sph_simulation::load_settings(fluid_file_name, parameters_file_name)."""
    return settings_from_dicts(read_property_file(fluid_file), read_property_file(params_file))


# The reference's property files, as numbers (fluid_properties/water.json,
# simulation_properties/default.json).
WATER = {"fluid_density": 998.29, "dynamic_viscosity": 3.5, "restitution": 0, "k": 100,
         "surface_tension_threshold": 7.065, "surface_tension": 0.0728,
         "particles_inside_influence_radius": 20}
DEFAULT_SIM = {"particles_count": 32000, "particle_mass": 0.05, "simulation_time": 10,
               "target_fps": 60, "simulation_scale": 0.1, "write_all_frames": False,
               "serialize": False, "constant_acceleration": {"x": 0, "y": -9.8, "z": 0}}
