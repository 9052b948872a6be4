"""Radargram output: drop-in for ``src/PYTHON/output_handling.py``.

``compile_rdrgrm`` (output_handling.py:4-34), ``get_simulation_range``
(:37-49), ``load_params`` (:52-72), ``load_attenuation_geom`` (:74-95) and
``roll_rdrgrm`` (:97-103) keep the reference's signatures and behaviour.
``save_radargram`` / ``load_radargram`` add a single-file complex64 binary
format (one ``.npy``) for the file-free path.
"""
import glob
import pickle

import numpy as np


def compile_rdrgrm(path, par, rx_win_file=None):
    """Stack ``s*.txt`` trace files into a complex (nr, ns) radargram."""
    filenames = glob.glob(f"{path}/s*.txt")
    if len(filenames) == 0:
        raise ValueError(f"No files found in {path} with pattern s*.txt")
    filenames.sort()
    if rx_win_file:
        rx_win_adj = np.load(rx_win_file)
        rx_win_adj_rb = (rx_win_adj - np.min(rx_win_adj)) // ((1 / par["rx_sample_rate"]) * 299792458)
        rx_win_adj_rb = rx_win_adj_rb.astype(int)
    rdrgrm = []
    for i, f in enumerate(filenames):
        if i < par["ns"]:
            index = int(f.split("/")[-1][1:-4])
            arr = np.loadtxt(f).T
            col = arr[0] + 1j * arr[1]
            if rx_win_file:
                col = np.roll(col, rx_win_adj_rb[index])
            rdrgrm.append(col)
    return np.array(rdrgrm).T


def get_simulation_range(path):
    filenames = sorted(glob.glob(f"{path}/s*.txt"))
    indices = [int(f.split("/")[-1][1:-4]) for f in filenames]
    return np.min(indices), np.max(indices)


def load_params(param_path, target_path, source_path=None):
    with open(param_path, "rb") as hdl:
        params = pickle.load(hdl)
    targets = np.genfromtxt(target_path, delimiter=",")
    if len(targets.shape) > 1:
        print("Multiple targets detected. Just using the first")
        targets = targets[0]
    params["tx"] = targets[0]
    params["ty"] = targets[1]
    params["tz"] = targets[2]
    if source_path:
        source_coords = np.genfromtxt(source_path, delimiter=",")
        params["ns"] = source_coords.shape[0]
    return params


def load_attenuation_geom(filepath):
    xmins, xmaxs, ymins, ymaxs, zmins, zmaxs, conductivities = [], [], [], [], [], [], []
    with open(filepath, "r") as f:
        for line in f:
            vals = line.strip().split(",")
            conductivities.append(float(vals[0]))
            xmins.append(float(vals[1]))
            ymins.append(float(vals[2]))
            zmins.append(float(vals[3]))
            xmaxs.append(float(vals[4]))
            ymaxs.append(float(vals[5]))
            zmaxs.append(float(vals[6]))
    return (conductivities, xmins, xmaxs, ymins, ymaxs, zmins, zmaxs)


def roll_rdrgrm(rdrgrm, shifts):
    corrected = np.zeros_like(rdrgrm)
    for i, shift in enumerate(shifts.astype(int)):
        corrected[:, i] = np.roll(rdrgrm[:, i], -1 * shift)
    return corrected


def save_radargram(path, rdrgrm):
    """Write a complex64 (nr, ns) radargram as one ``.npy`` file."""
    np.save(path, np.asarray(rdrgrm, dtype=np.complex64))


def load_radargram(path):
    return np.load(path)
