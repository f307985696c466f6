"""An independent reading of PrefabAsset::Spawn (Sources/Asset/PrefabAsset.cpp:30-120)
in Python, for the asset-loader tests and the fixture generator: entity
graph from the .pf JSON (nested Instance prefabs included), world matrices
from a caller-supplied RealculateMatrix (the reference's own, compiled by
oracle/ref/build_ref.py). Test infrastructure."""
import json
import os

import numpy as np


def fnv1a64(s):
    h = 14695981039346656037
    for c in s.encode():
        h ^= c
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def guid_index(mods_dir):
    idx = {}
    for root, _, files in os.walk(mods_dir):
        for f in files:
            full = os.path.join(root, f)
            rel = os.path.relpath(full, mods_dir).replace(os.sep, "/")
            idx[fnv1a64(rel)] = full
    return idx


def _vec3(s):
    return np.array([float(x) for x in s.split(" ")[:3]], np.float32)


def spawn(mods_dir, mod_path, realculate):
    """-> list of renderers (world16, pivot3, vox_guid, pal_guid) in creation order."""
    idx = guid_index(mods_dir)
    ents = []  # dict(parent, pos, rot, scale, vox, pal, pivot)

    def go(path, parent_entity):
        doc = json.load(open(path))
        id_map = {}
        root = None
        for ent in doc:
            parent = id_map.get(ent["Parent"]) if ent.get("Parent") is not None else None
            is_root = parent is None
            if ent.get("Instance") is not None:
                e = go(idx[int(ent["Instance"], 16)], parent)
            else:
                e = len(ents)
                ents.append(dict(parent=None, pos=np.zeros(3, np.float32), rot=np.zeros(3, np.float32),
                                 scale=np.ones(3, np.float32), vox=0, pal=0, pivot=np.zeros(3, np.float32)))
            id_map[ent["Id"]] = e
            if is_root:
                root = e
                ents[e]["parent"] = parent_entity
            else:
                ents[e]["parent"] = parent
            tr = ent.get("Transform")
            if tr is not None:
                ents[e]["pos"] = _vec3(tr["Position"])
                ents[e]["rot"] = _vec3(tr["Rotation"])
                ents[e]["scale"] = _vec3(tr["Scale"])
            vr = ent.get("VoxRenderer")
            if vr is not None:
                ents[e]["vox"] = int(vr["Vox"], 16)
                ents[e]["pal"] = int(vr["Pallete"], 16)
                if vr.get("Pivot") is not None:
                    ents[e]["pivot"] = _vec3(vr["Pivot"])
        return root

    go(idx[fnv1a64(mod_path)], None)
    world = [None] * len(ents)

    def w(i):
        if world[i] is None:
            p = ents[i]["parent"]
            world[i] = realculate(ents[i]["pos"], ents[i]["rot"], ents[i]["scale"], None if p is None else w(p))
        return world[i]

    out = []
    for i, e in enumerate(ents):
        if e["vox"]:
            out.append((w(i), e["pivot"], e["vox"], e["pal"], idx))
    return out
