"""Parameter generation: drop-in for the reference's ``src/PYTHON/param_gen.py``.

Same call signatures and dictionary keys as the reference
(``gen_params`` param_gen.py:17-129, ``export_params`` :4-14,
``vert_source_path`` :131-144, ``track_Z_rxwin`` :146-152), plus
``to_rp_params`` which turns a parameter dictionary into the ``rp_params``
struct of the C ABI the way ``parseSimulationParameters``
(src/CUDA/file_io.cu:122-249) reads a JSON file: the same required keys, the
same defaults, and a ``KeyError`` naming the key when a required one is
missing.
"""
import json
import pickle

import numpy as np

from . import _abi

# Instrument presets (param_gen.py:45-67).
PLATFORMS = {
    "REASON_VHF": dict(power=100, frequency=60e6, bandwidth=10e6, surface_gain=7.3),
    "REASON_HF": dict(power=100, frequency=9e6, bandwidth=1e6, surface_gain=4.0),
    "1MHz": dict(power=100, frequency=1e6, bandwidth=1e5, surface_gain=4.0),
}

# Media presets (param_gen.py:70-79).
MEDIA = {
    "planetary_ice": dict(eps_2=3.15, sig_2=1e-6, rms_height=0.4),
    "vacuum": dict(eps_2=1.0, sig_2=0, rms_height=0),
}


def export_params(params, filename, directory="inputs"):
    """Write ``{directory}/{filename}.json`` and ``.pkl`` (param_gen.py:4-14)."""
    for k in params.keys():
        if params[k] is None:
            raise ValueError(f"Found null for key [{k}] when exporting parameter dict")
    with open(f"{directory}/{filename}.json", "w") as f:
        json.dump(params, f, indent=4)
    with open(f"{directory}/{filename}.pkl", "wb") as hdl:
        pickle.dump(params, hdl, protocol=pickle.HIGHEST_PROTOCOL)


def gen_params(platform, media, domainpar, recpar, sourcepar, par=None):
    """Build a parameter dictionary (param_gen.py:17-129)."""
    pars = {}
    pars["eps_1"] = 1.0
    pars["sig_1"] = 0.0
    pars["mu_1"] = 1.0
    pars["mu_2"] = 1.0
    pars["convolution"] = True
    pars["convolution_linear"] = True
    pars["specular"] = False
    pars["lossless"] = False
    pars["incoherent"] = False
    pars["debug_surface"] = False
    pars["rerad_funct"] = 2
    pars["buff"] = 1.1
    if platform not in PLATFORMS:
        raise ValueError(f"platform {platform} not recognized.")
    inst = PLATFORMS[platform]
    pars["power"] = inst["power"]
    pars["frequency"] = inst["frequency"]
    pars["bandwidth"] = inst["bandwidth"]
    pars["surface_gain"] = inst["surface_gain"]
    pars["subsurface_gain"] = pars["surface_gain"]
    pars["polarization"] = "HH"
    if media not in MEDIA:
        raise ValueError(f"media {media} not recognized.")
    med = MEDIA[media]
    pars["eps_2"] = med["eps_2"]
    pars["sig_2"] = med["sig_2"]
    pars["rms_height"] = med["rms_height"]
    if "fs" not in domainpar.keys():
        raise ValueError("Facet size (fs) missing from input dictionary domainpar")
    pars["fs"] = domainpar["fs"]
    if "ox" in domainpar.keys():
        print("Parameter generation detected simple surface type domain inputs. "
              "Adding to parameter dict.")
        for k in domainpar.keys():
            if k not in pars.keys():
                pars[k] = domainpar[k]
    for k in ("rx_window_m", "rx_sample_rate"):
        if k not in recpar.keys():
            raise ValueError(f"key {k} neccessary in recpar which has keys {recpar.keys()}")
        pars[k] = recpar[k]
    if "rx_window_position_file" in recpar.keys():
        pars["rx_window_position_file"] = recpar["rx_window_position_file"]
    if "rx_window_offset_m" in recpar.keys():
        pars["rx_window_offset_m"] = recpar["rx_window_offset_m"]
    if "rx_window_position_file" not in recpar.keys() and "rx_window_offset_m" not in recpar.keys():
        raise ValueError("input dictionary recpar needs either a rx window position file "
                         "or a static rx window offset")
    for k in ("ns", "aperture"):
        if k not in sourcepar.keys():
            raise ValueError(f"key {k} necessary in sourcepar which has keys {sourcepar.keys()}")
        pars[k] = sourcepar[k]
    if "source_path_file" in sourcepar.keys():
        pars["source_path_file"] = sourcepar["source_path_file"]
    else:
        for lk in ("sx0", "sy", "sz", "sdx"):
            pars[lk] = sourcepar[lk]
    if par is not None:
        for k in par.keys():
            pars[k] = par[k]
    pars["lam"] = 299792458 / pars["frequency"]
    pars["k"] = (2 * np.pi) / pars["lam"]
    if "sz" in pars.keys():
        pars["altitude"] = pars["sz"]
    return pars


def vert_source_path(params, minZ, maxZ, filename, direct="inputs", xoff=0, yoff=0):
    """Vertical source path file (param_gen.py:131-144)."""
    sz = np.linspace(minZ, maxZ, params["ns"])
    sy = np.zeros_like(sz) + yoff
    sx = np.zeros_like(sz) + xoff
    with open(f"{direct}/{filename}.txt", "w") as f:
        for i in range(params["ns"]):
            sep = "" if i == params["ns"] - 1 else "\n"
            f.write(f"{sx[i]},{sy[i]},{sz[i]}{sep}")
    return sz


def track_Z_rxwin(sz, ahead, filename, direct="inputs"):
    """Receive-window position file (param_gen.py:146-152)."""
    rx_window_positions = sz - ahead
    with open(f"{direct}/{filename}.txt", "w") as f:
        for pos in rx_window_positions:
            f.write(f"{pos}\n")


_REQUIRED = ("frequency", "bandwidth", "power", "aperture", "rms_height", "buff",
             "eps_1", "eps_2", "sig_1", "sig_2", "rx_sample_rate", "rx_window_m", "fs",
             "rerad_funct", "convolution", "convolution_linear", "specular", "lossless")


def _req(j, key):
    if key not in j:
        raise KeyError(f"required parameter '{key}' missing")
    return j[key]


def to_rp_params(j, derive=True):
    """Parameter dict (the JSON of ``export_params``) -> derived ``RpParams``.

    Mirrors parseSimulationParameters (src/CUDA/file_io.cu:122-249): keys read
    with ``j[...]`` there are required here, keys read with ``j.value(...)``
    take the same defaults.  Derived constants come from the library's
    ``rp_params_derive``.
    """
    p = _abi.RpParams()
    for key in _REQUIRED:
        _req(j, key)
    p.frequency = float(j["frequency"])
    p.bandwidth = float(j["bandwidth"])
    p.power = float(j["power"])
    p.aperture = float(j["aperture"])
    if j.get("gain_pattern_file", "NONE") == "NONE":
        p.subsurface_gain = float(_req(j, "subsurface_gain"))
        p.surface_gain = float(_req(j, "surface_gain"))
    p.rms_height = float(j["rms_height"])
    p.buff = float(j["buff"])
    p.eps_1 = float(j["eps_1"])
    p.eps_2 = float(j["eps_2"])
    p.sig_1 = float(j["sig_1"])
    p.sig_2 = float(j["sig_2"])
    p.rx_sample_rate = float(j["rx_sample_rate"])
    p.rx_window_m = float(j["rx_window_m"])
    if j.get("rx_window_position_file", "NONE") == "NONE":
        p.rx_window_offset_m = float(_req(j, "rx_window_offset_m"))
    p.fs = float(j["fs"])
    p.source_normal_multiplier = float(j.get("source_normal_multiplier", 1.0))
    p.altitude = float(j.get("altitude", 0.0))
    if j.get("source_path_file", "NONE") == "NONE":
        p.sy = float(_req(j, "sy"))
        p.sz = float(_req(j, "sz"))
        p.sx0 = float(_req(j, "sx0"))
        p.sdx = float(_req(j, "sdx"))
        p.ns = int(_req(j, "ns"))
    elif "ns" in j:
        p.ns = int(j["ns"])
    p.rerad_funct = int(j["rerad_funct"])
    p.convolution = int(bool(j["convolution"]))
    p.convolution_linear = int(bool(j["convolution_linear"]))
    p.specular = int(bool(j["specular"]))
    p.lossless = int(bool(j["lossless"]))
    p.incoherent = int(bool(j.get("incoherent", False)))
    p.incoherent_seed = int(j.get("incoherent_seed", 1))      # extension: seeded incoherent phases
    p.disable_surface = int(bool(j.get("disable_surface", False)))
    p.debug_surface = int(bool(j.get("debug_surface", False)))
    p.pol = 0
    if derive:
        _abi.check("rp_params_derive", _abi.lib().rp_params_derive(_byref(p)))
    return p


def _byref(p):
    import ctypes
    return ctypes.byref(p)
