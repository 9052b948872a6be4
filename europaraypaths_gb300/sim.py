"""Command-line drop-in for the reference's ``sim`` program.

    python -m europaraypaths_gb300.sim params.json facets.fct targets.txt outdir [--form auto|fast|plain]

Same arguments, JSON keys and input files as ``src/CUDA/sim.cu`` (main,
sim.cu:92-1052): the parameter file (parseSimulationParameters), the facet
and target files, and the optional source-path, gain-pattern, receive-window
and attenuation-geometry files named in the JSON.  Writes ``outdir/s%06d.txt``
("%e %e" per range bin) for every trace that illuminates at least one facet,
after removing old ``s*.txt`` files, and prints the run summary with
traces/s.  Facet and target inputs may also be binary stores (detected by
their header); ``--radargram PATH`` writes every trace into one radargram
file instead of the text files.  Errors are reported with a non-zero exit status instead of an
abort.  ``debug_surface`` dumps are not produced.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

from . import _abi, fileio, param_gen, traces as tr_mod


def load_inputs(params_path, facets_path, targets_path):
    """Parse every input the reference's main() reads; returns
    (rp_params, facets (12,N), targets (7,T), prisms (7,P) or None, traces (ns,9))."""
    fileio_check = fileio.count_records   # noqa: F841  (library must load first)
    if not os.path.isfile(params_path):
        raise _abi.RaypathError("parseSimulationParameters", -2, f"File not found: {params_path}")
    with open(params_path) as f:
        j = json.load(f)
    p = param_gen.to_rp_params(j)
    src_file = j.get("source_path_file", "NONE")
    if src_file != "NONE":
        sources = fileio.read_sources(src_file)
        ns = sources.shape[0]
    else:
        sources = None
        ns = p.ns
    gains = None
    gfile = j.get("gain_pattern_file", "NONE")
    if gfile != "NONE":
        gains = fileio.read_gains(gfile)
        if gains.shape[0] != ns:
            print(f"ERROR: Gain pattern file has {gains.shape[0]} lines, but number of sources is {ns}",
                  file=sys.stderr)
            gains = np.resize(gains, (ns, 2))
    rx = None
    rfile = j.get("rx_window_position_file", "NONE")
    if rfile != "NONE":
        rx = fileio.read_rx_window(rfile, ns)
    targets = fileio.load_targets(targets_path)
    facets = fileio.load_facets(facets_path)
    prisms = None
    afile = j.get("attenuation_geometry_file", "NONE")
    if afile != "NONE":
        prisms = fileio.read_prisms(afile, p)
    if sources is None:
        tr = tr_mod.linear_track(p, ns)
        if rx is not None:
            tr[:, 6] = rx
        if gains is not None:
            tr[:, 7] = np.power(10.0, gains[:, 0] / 10.0)
            tr[:, 8] = np.power(10.0, gains[:, 1] / 10.0)
    else:
        tr = tr_mod.from_sources(p, sources, rx_window=rx, gains_db=gains)
    return p, facets, targets, prisms, tr


def pick_form(p, targets):
    """``auto``: the fast form, which runs every mode the reference defines
    (the default mode; specular with linear, circular or no convolution;
    targets of either type).  ``plain`` selects the FP64 form explicitly."""
    return "fast"


def run(params_path, facets_path, targets_path, outdir, form="auto", batch=64, quiet=False, radargram=None):
    t0 = time.perf_counter()
    fileio.check_directory(outdir)
    p, facets, targets, prisms, tr = load_inputs(params_path, facets_path, targets_path)
    if form == "auto":
        form = pick_form(p, np.asarray(targets).reshape(7, -1))
    from .simulator import Scene
    scene = Scene(p, facets, targets, prisms=prisms)
    ns = tr.shape[0]
    written = 0
    if radargram is not None:
        rdr = np.zeros((ns, scene.nr), np.complex64)
    else:
        fileio.clear_traces(outdir)
    for s0 in range(0, ns, batch):
        out, counts = scene.simulate(tr[s0:s0 + batch], form=form, return_counts=True)
        if radargram is not None:      # every trace, zero where nothing is illuminated
            rdr[s0:s0 + out.shape[0]] = out
            written += int(np.count_nonzero(counts[:, 0]))
            continue
        for k in range(out.shape[0]):
            if counts[k, 0] == 0:
                if not quiet:
                    print(f"No illuminated facets for source {s0 + k}, skipping.")
                continue
            fileio.write_trace(os.path.join(outdir, f"s{s0 + k:06d}.txt"), out[k])
            written += 1
    scene.close()
    if radargram is not None:
        fileio.write_radargram(radargram, rdr)
    dt = time.perf_counter() - t0
    if not quiet:
        print("=== Run summary ===")
        print(f"Total runtime: {dt:.3f} s")
        if ns > 0:
            print(f"Time per source (trace): {1e3 * dt / ns:.3f} ms ({dt / ns:.6f} s)")
            print(f"Throughput: {ns / dt:.2f} traces/sec")
    return written


def main(argv=None):
    ap = argparse.ArgumentParser(prog="sim", description=__doc__.splitlines()[0])
    ap.add_argument("params")
    ap.add_argument("facets")
    ap.add_argument("targets")
    ap.add_argument("outdir")
    ap.add_argument("--form", default="auto", choices=["auto", "fast", "plain"])
    ap.add_argument("--batch", type=int, default=64, help="traces per engine call")
    ap.add_argument("--radargram", default=None, help="write one radargram file (all traces) instead of s*.txt")
    a = ap.parse_args(argv)
    try:
        run(a.params, a.facets, a.targets, a.outdir, form=a.form, batch=a.batch, radargram=a.radargram)
    except (_abi.RaypathError, KeyError, ValueError) as e:
        print(f"sim: {e}", file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
