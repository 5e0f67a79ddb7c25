"""Vp/Vs SU models of the reference's example input folders (tests/golden/inputs/<case>/).

The reference generates them with MATLAB (examples/test1/input/create_one_layer_model.m,
examples/test2/input/create_two_layers_model.m:19-34, examples/test3/input/create_three_layers_model.m,
examples/test4/input/create_two_layers_model.m:31-39); this restates those layer geometries:
(nz + npml) x (nx + 2 npml) cells at the example's dx, dz, with layer j from row round(h_j/dz) + 1
down (1-based); test4 puts its Moho at 35 km under the first fix(NX/2) columns and at 30 km under
the rest.  The Altyn example's smoothed models are not in the reference tree; it gets a stand-in:
its left FK model's layers under the left half of the profile and its right FK model's under the
right half.  Files: one 240-byte header (zeros) and NZ float32 samples per trace, NX traces.
"""
import os
import shutil

import numpy as np

GOLDEN_INPUTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "inputs")
CASES = ("test1", "test2", "test3", "test4", "Altyn")

# (vp, vs, top depth in m) per layer, as the create_*.m scripts set them
LAYERS = {
    "test1": [(6000.0, 3450.0, 0.0)],
    "test2": [(6000.0, 3450.0, 0.0), (8000.0, 4450.0, 35e3)],
    "test3": [(6000.0, 3450.0, 0.0), (8000.0, 4450.0, 30e3), (7200.0, 4000.0, 100e3)],
    "test4": [(6000.0, 3450.0, 0.0), (8000.0, 4450.0, 35e3)],
}


def _numbers(line):
    return [float(t.replace("d", "e").replace("D", "e")) for t in line.replace(",", " ").split()]


def read_fd_model(folder):
    lines = open(os.path.join(folder, "FD_model.dat")).read().splitlines()
    x0, xn, z0, zn, dx, dz, _ = _numbers(lines[3])[:7]
    tok = lines[5].replace(",", " ").split()
    npml = int(tok[2])
    return dict(nx=int(round((xn - x0) / dx)) + 1, nz=int(round((zn - z0) / dz)) + 1, npml=npml, dx=dx, dz=dz)


def read_fk_layers(folder, name):
    lines = open(os.path.join(folder, name)).read().splitlines()
    n = int(_numbers(lines[1])[0])
    return [tuple(_numbers(lines[3 + i])[:3]) for i in range(n)]


def _fill(vp, vs, layers, dz, cols):
    for v_p, v_s, top in layers:
        ih = int(round(top / dz))
        vp[ih:, cols] = v_p
        vs[ih:, cols] = v_s


def models(case, folder):
    g = read_fd_model(folder)
    NZ, NX = g["nz"] + g["npml"], g["nx"] + 2 * g["npml"]
    vp = np.zeros((NZ, NX), np.float32)
    vs = np.zeros((NZ, NX), np.float32)
    if case == "test4":
        nx0 = NX // 2
        _fill(vp, vs, LAYERS["test4"], g["dz"], slice(0, nx0))
        _fill(vp, vs, [(6000.0, 3450.0, 0.0), (8000.0, 4450.0, 30e3)], g["dz"], slice(nx0, NX))
    elif case in LAYERS:
        _fill(vp, vs, LAYERS[case], g["dz"], slice(0, NX))
    else:
        half = NX // 2
        _fill(vp, vs, read_fk_layers(folder, "FK_model_left.dat"), g["dz"], slice(0, half))
        _fill(vp, vs, read_fk_layers(folder, "FK_model_right.dat"), g["dz"], slice(half, NX))
    return vp, vs


def write_su_model(path, v):
    head = np.zeros(120, np.int16).tobytes()
    with open(path, "wb") as f:
        for ix in range(v.shape[1]):
            f.write(head)
            f.write(np.ascontiguousarray(v[:, ix], np.float32).tobytes())


def make_case(case, dst, fd_edit=None):
    """Copies the case's input folder to dst, writes its Vp/Vs models there, returns the folder.
    fd_edit(lines) may change FD_model.dat's lines (e.g. a shorter record)."""
    src = os.path.join(GOLDEN_INPUTS, case)
    shutil.copytree(src, dst)
    if fd_edit is not None:
        p = os.path.join(dst, "FD_model.dat")
        lines = open(p).read().splitlines()
        open(p, "w").write("\n".join(fd_edit(lines)) + "\n")
    names = [l.strip() for l in open(os.path.join(dst, "inpar.dat")).read().splitlines() if l.strip()]
    vp, vs = models(case, dst)
    write_su_model(os.path.join(dst, names[5]), vp)
    write_su_model(os.path.join(dst, names[6]), vs)
    return dst
