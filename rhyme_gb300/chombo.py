"""Chombo-layout level output written without HDF5.

The reference writes its snapshots with HDF5 (rhyme_chombo_write_samr.f90,
_write_headers.f90:3-65, _write_level_data.f90:3-72). libhdf5 is not
available to this project, so a snapshot is stored as one flat container
holding the same objects: the header attributes (ProblemDomain, num_levels,
num_components, component_<i> labels, iteration, time, Chombo_global
SpaceDim and unit strings), and per level its dx, ref_ratio, prob_domain,
`boxes` table (lo_i lo_j lo_k hi_i hi_j hi_k, int32) and `data:datatype=0`
(FP32). A converter to HDF5 needs only to copy these objects.

Container: b"RHYMECHOMBO1\\n", an 8-byte little-endian header length, the
header as JSON, then for each level its boxes table and its data, each as
raw little-endian arrays at the offsets the header gives.
"""
import json

import numpy as np

MAGIC = b"RHYMECHOMBO1\n"


def level_length(dims_list, ncmp):
    return int(sum(int(np.prod(d)) for d in dims_list)) * int(ncmp)


def write(path, levels, attrs):
    """levels: list of dicts with keys dx (3 floats), ref_ratio, boxes
    ((n, 6) int32), data (float32); attrs: header attributes."""
    header = {"attrs": attrs, "levels": []}
    blobs = []
    off = 0
    for lv in levels:
        boxes = np.ascontiguousarray(lv["boxes"], dtype="<i4")
        data = np.ascontiguousarray(lv["data"], dtype="<f4")
        entry = {"dx": [float(x) for x in lv["dx"]], "ref_ratio": int(lv.get("ref_ratio", 2)),
                 "prob_domain": [int(x) for x in lv.get("prob_domain", [0] * 6)],
                 "boxes": {"offset": off, "shape": list(boxes.shape)}}
        off += boxes.nbytes
        entry["data:datatype=0"] = {"offset": off, "length": int(data.size)}
        off += data.nbytes
        header["levels"].append(entry)
        blobs += [boxes, data]
    hb = json.dumps(header).encode()
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(np.uint64(len(hb)).astype("<u8").tobytes())
        f.write(hb)
        for b in blobs:
            f.write(b.tobytes())


def read(path):
    with open(path, "rb") as f:
        if f.read(len(MAGIC)) != MAGIC:
            raise ValueError("%s is not a Chombo-layout container" % path)
        n = int(np.frombuffer(f.read(8), dtype="<u8")[0])
        header = json.loads(f.read(n).decode())
        raw = f.read()
    levels = []
    for e in header["levels"]:
        bo, shp = e["boxes"]["offset"], e["boxes"]["shape"]
        boxes = np.frombuffer(raw, dtype="<i4", count=int(np.prod(shp)), offset=bo).reshape(shp)
        d = e["data:datatype=0"]
        data = np.frombuffer(raw, dtype="<f4", count=d["length"], offset=d["offset"])
        levels.append({"dx": e["dx"], "ref_ratio": e["ref_ratio"], "prob_domain": e["prob_domain"],
                       "boxes": boxes, "data": data})
    return header["attrs"], levels


def header_attrs(ndim, base_grid, labels, iteration, time, units=None):
    """The root and Chombo_global attributes of
    rhyme_chombo_write_headers.f90:23-63."""
    pd = list(base_grid) + [1] * (3 - len(base_grid))
    attrs = {"ProblemDomain": pd, "num_levels": 1, "num_components": len(labels),
             "iteration": int(iteration), "time": float(time),
             "Chombo_global": dict({"SpaceDim": 3}, **(units or {}))}
    for i, lab in enumerate(labels):
        attrs["component_%d" % i] = lab
    return attrs
