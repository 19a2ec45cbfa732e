"""On-disk formats of the reference driver, byte-compatible.

* v4 particle snapshot ``particles_NNNNN.bin`` (reference
  ``src/main.cpp:2132-2202`` writer, ``:2010-2126`` reader,
  ``include/ParticleSystem.hpp:1204-1220`` magic/version/endian): an 88-byte
  header (``KPTPRT\\0\\0``, u32 version 4, u32 endian marker 0x01020304, i32
  space_dim, i32 species, u64 count, u64 capacity, f64 rest_mass, charge,
  speed_of_light, energy_scale_erg, split_ratio, minimum_child_weight) then
  100-byte records (u64 id, i32 status, i32 split_level, i32 sort_key,
  f64 position[2], previous_position[2], previous_step_position[2], p, mu,
  weight, initial_kinetic_energy).
* momentum histogram CSV (``src/main.cpp:1942-1963``): header
  ``bin,p_left,p_right,weight`` and values printed with 16 significant
  digits.
* summary CSV (``src/main.cpp:2207-2235``): 22 columns.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List

import numpy as np

MAGIC = b"KPTPRT\x00\x00"
VERSION = 4
ENDIAN_MARKER = 0x01020304
HEADER_BYTES = 88
RECORD_DTYPE = np.dtype([
    ("id", "<u8"), ("status", "<i4"), ("split_level", "<i4"), ("sort_key", "<i4"),
    ("position", "<f8", (2,)), ("previous_position", "<f8", (2,)),
    ("previous_step_position", "<f8", (2,)), ("p", "<f8"), ("mu", "<f8"), ("weight", "<f8"),
    ("initial_kinetic_energy", "<f8")])
assert RECORD_DTYPE.itemsize == 100

SUMMARY_COLUMNS = ("frame,time,stored,active,inactive,weight_sum,p_min,p_max,p_avg,dt_min,"
                   "dt_max,dt_avg,max_split_level,injected,split,skipped_split_capacity,"
                   "read_seconds,inject_seconds,move_seconds,split_seconds,"
                   "total_frame_seconds,total_elapsed_seconds").split(",")


@dataclasses.dataclass
class Snapshot:
    space_dim: int
    species: int
    count: int
    capacity: int
    rest_mass: float
    charge: float
    speed_of_light: float
    energy_scale_erg: float
    split_ratio: float
    minimum_child_weight: float
    records: np.ndarray

    def to_arrays(self) -> Dict[str, np.ndarray]:
        """Driver SoA arrays (time and step size are not stored: zeros)."""
        r = self.records
        return {"x": r["position"][:, 0].copy(), "y": r["position"][:, 1].copy(),
                "p": r["p"].copy(), "t": np.zeros(self.count), "dt": np.zeros(self.count),
                "w": r["weight"].copy(), "mu": r["mu"].copy(),
                "status": r["status"].astype(np.int32), "level": r["split_level"].astype(np.int32)}


def read_snapshot(path: str) -> Snapshot:
    raw = open(path, "rb").read()
    if len(raw) < HEADER_BYTES or raw[:8] != MAGIC:
        raise ValueError("Restart particle snapshot is not a repository KPTPRT file.")
    head = np.frombuffer(raw[8:HEADER_BYTES], dtype=np.uint8)
    version, endian = head[:8].view("<u4")
    if version != VERSION:
        raise ValueError("Restart particle snapshot must use particle binary version 4.")
    if endian != ENDIAN_MARKER:
        raise ValueError("Restart particle snapshot endian does not match this host.")
    space_dim, species = head[8:16].view("<i4")
    count, capacity = head[16:32].view("<u8")
    doubles = head[32:80].view("<f8")
    body = raw[HEADER_BYTES:]
    if len(body) < int(count) * RECORD_DTYPE.itemsize:
        raise ValueError("Failed to read particle binary scalar.")
    records = np.frombuffer(body[: int(count) * RECORD_DTYPE.itemsize], dtype=RECORD_DTYPE)
    return Snapshot(int(space_dim), int(species), int(count), int(capacity), *map(float, doubles),
                    records=records.copy())


def write_snapshot(path: str, arrays: Dict[str, np.ndarray], count: int, capacity: int,
                   charge: float, split_ratio: float, p0: float) -> None:
    """The driver's snapshot writer (src/main.cpp:2132-2202)."""
    header = bytearray(MAGIC)
    header += np.array([VERSION, ENDIAN_MARKER], dtype="<u4").tobytes()
    header += np.array([2, 3], dtype="<i4").tobytes()
    header += np.array([count, capacity], dtype="<u8").tobytes()
    header += np.array([1.0, charge, 1.0, 1.0, split_ratio, 0.0], dtype="<f8").tobytes()
    rec = np.zeros(count, dtype=RECORD_DTYPE)
    rec["id"] = np.arange(count, dtype=np.uint64)
    rec["status"] = arrays["status"][:count]
    rec["split_level"] = arrays["level"][:count]
    pos = np.stack([arrays["x"][:count], arrays["y"][:count]], axis=1)
    rec["position"] = pos
    rec["previous_position"] = pos
    rec["previous_step_position"] = pos
    rec["p"] = arrays["p"][:count]
    rec["mu"] = arrays["mu"][:count]
    rec["weight"] = arrays["w"][:count]
    rec["initial_kinetic_energy"] = math.sqrt(1.0 + p0 * p0) - 1.0
    with open(path, "wb") as stream:
        stream.write(bytes(header))
        stream.write(rec.tobytes())


def format_g16(value: float) -> str:
    """``std::setprecision(16)`` default float formatting (%.16g)."""
    return "%.16g" % value


def histogram_edges(pmin: float, pmax: float, nbins: int) -> List[tuple]:
    """(p_left, p_right) per bin as the driver computes them (src/main.cpp:1952-1957)."""
    dlogp = (math.log(pmax) - math.log(pmin)) / nbins
    return [(math.exp(math.log(pmin) + b * dlogp), math.exp(math.log(pmin) + (b + 1) * dlogp))
            for b in range(nbins)]


def write_histogram_csv(path: str, bins: np.ndarray, pmin: float, pmax: float) -> None:
    with open(path, "w") as stream:
        stream.write("bin,p_left,p_right,weight\n")
        for b, (left, right) in enumerate(histogram_edges(pmin, pmax, len(bins))):
            stream.write(f"{b},{format_g16(left)},{format_g16(right)},{format_g16(bins[b])}\n")


def read_histogram_csv(path: str) -> Dict[str, np.ndarray]:
    rows = [line.strip().split(",") for line in open(path) if line.strip()]
    if rows[0] != ["bin", "p_left", "p_right", "weight"]:
        raise ValueError("not a momentum histogram CSV")
    data = np.array([[float(v) for v in r] for r in rows[1:]])
    return {"bin": data[:, 0].astype(int), "p_left": data[:, 1], "p_right": data[:, 2],
            "weight": data[:, 3]}


def read_summary_csv(path: str) -> List[Dict[str, str]]:
    lines = [line.rstrip("\n") for line in open(path) if line.strip()]
    header = lines[0].split(",")
    if header != list(SUMMARY_COLUMNS):
        raise ValueError("not a reconnection summary CSV")
    return [dict(zip(header, line.split(","))) for line in lines[1:]]
