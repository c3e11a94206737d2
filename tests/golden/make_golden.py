"""Generate the golden fixtures in tests/golden/ from the reference's own C.

Run here (where the reference checkout exists):

    python tests/golden/make_golden.py --ref <reference checkout>   (or set EDMD_REFERENCE_DIR)

It builds ``oracle/_ref/ref_trace`` (``make -C oracle ref``), which compiles
the reference's unmodified src/EDMD.c and satellites with IEEE flags and
re-runs its main loop (src/EDMD.c:523-618) with a trace hook, then stores
for each case:

* the initial state after the reference's own init (src/EDMD.c:1356-1839,
  normalizePhysicalQ 5723-5764),
* every accepted collision ``(i, j, cell_i, cell_j, t)`` in processing order,
* the collision-virial accumulators, final time and counters,
* the state after free-flying every disk to the final time.

The fixtures are what the GPU parity tests compare against; the tests read
only these files, never the reference checkout.
"""
import argparse
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# name: (reference CLI args, max accepted collisions, keep full final state)
CASES = {
    "hex2000_v1": ("--hex -N 2000 --phi 0.70 -x 0 -v 1", 10000, True),
    "hex2000_v2": ("--hex -N 2000 --phi 0.70 -x 0 -v 2", 10000, True),
    "hex1024_v3": ("--hex -N 1024 --phi 0.60 -x 0 -v 3", 10000, True),
    "hex10000_v4": ("--hex -N 10000 --phi 0.72 -x 0 -v 4", 10000, False),
    "grow256_v7": ("-N 256 --phi 0.5 -x 0.5 -q 0.7142857 -v 7", 20000, True),
    "grow400_v11": ("-N 400 --phi 0.74 -x 0.5 -q 0.7142857 -v 11", 20000, True),
    "grow300_v5": ("-N 300 --phi 0.3 -x 0.5 -q 0.7142857 -v 5", 20000, True),
}

# boxes of four to five cells a side, where the 3x3 neighbourhood of a cell
# wraps onto the cells at its other side
TINY_CASES = {
    "tiny_hex12": ("--hex -N 12 --phi 0.4 -x 0 -v 3", 3000, True),
    "tiny_grow10": ("-N 10 --phi 0.3 -x 0.5 -q 0.7 -v 3", 3000, True),
    "tiny_grow20": ("-N 20 --phi 0.5 -x 0.5 -q 0.7 -v 5", 3000, True),
}

# the command line's other physical options: restitution (-r), energy per
# disk (-E, the Hex velocities and the growth stop's normalisation) and box
# aspect ratio (-a)
OPTION_CASES = {
    "opt_res_hex": ("--hex -N 400 --phi 0.6 -x 0 -r 0.9 -v 2", 5000, True),
    "opt_einit_hex": ("--hex -N 400 --phi 0.6 -x 0 -E 2.5 -v 3", 5000, True),
    "opt_einit_grow": ("-N 300 --phi 0.6 -x 0.5 -q 0.7142857 -E 2.5 -v 6", 12000, True),
    "opt_aspect_grow": ("-N 300 --phi 0.55 -x 0.5 -q 0.7142857 -a 2.0 -v 8", 12000, True),
    "opt_aspect_hex": ("--hex -N 500 --phi 0.6 -x 0 -a 0.5 -v 9", 5000, True),
}

# runs the reference ends with its overlap abort (collisionTimeNormal,
# src/EDMD.c:2708-2717, exit(3)): the collisions before it and the pair it
# names are kept
ABORT_CASES = {
    "abort_hex8": "--hex -N 8 --phi 0.2 -x 0 -v 3",
    "abort_grow6": "-N 6 --phi 0.3 -x 0.5 -q 0.7 -v 4",
}

# the same kind of runs with additive contact, r1 + r2 (the reference's own
# switch NONADDITIVE set to 1 at src/EDMD.c:35; built by
# `make -C oracle ref-additive`); their fixtures carry contact = 1
ADDITIVE_CASES = {
    "add_grow256_v7": ("-N 256 --phi 0.5 -x 0.5 -q 0.7142857 -v 7", 20000, True),
    "add_grow400_v11": ("-N 400 --phi 0.74 -x 0.5 -q 0.7142857 -v 11", 20000, True),
    "add_grow300_v5": ("-N 300 --phi 0.3 -x 0.5 -q 0.4 -v 5", 20000, True),
}

# a short run whose dump and thermo files are kept verbatim (format pin)
FILES_CASE = ("files_hex64", "--hex -N 64 --phi 0.5 -x 0 -v 9 -t 1200 -D 100 -o 50")

# bidisperse growth starts whose dump and thermo files are kept verbatim, with
# the reference's contact rule and with additive contact (contact = 1: the
# drop-in program runs them with --additive)
FILES_GROW_CASES = {
    "files_grow64": ("-N 64 --phi 0.5 -x 0.5 -q 0.4 -v 9 -t 1100 -D 100 -o 25", 0),
    "files_add_grow64": ("-N 64 --phi 0.5 -x 0.5 -q 0.4 -v 9 -t 1100 -D 100 -o 25", 1),
}

# restarts with -l (src/EDMD.c:980-995, 1366-1451): from a .txt state (the
# final positions of the files case; velocities drawn anew) and from the
# last frame of the files case's dump (velocities kept); {golden} is this
# directory.  Their dump and thermo files are kept verbatim too.
LOAD_TXT = "load64.txt"
LOAD_CASES = {
    "load_txt64": "-l {golden}/load64.txt -t 1200 -D 100 -o 50 -v 9",
    "load_dump64": "-l {golden}/files_hex64.dump -t 1200 -D 100 -o 50 -v 9",
}


def hx(s):
    return float.fromhex(s)


def parse_trace(path):
    init, colls, state = [], [], []
    vir = tfin = None
    head = None
    with open(path) as f:
        for line in f:
            p = line.split()
            if p[0] == "#":
                head = dict(N=int(p[2]), Lx=hx(p[4]), Ly=hx(p[6]), Nxc=int(p[8]), Nyc=int(p[10]))
            elif p[0] == "I":
                init.append([hx(v) for v in p[2:8]] + [int(p[8])])
            elif p[0] == "C":
                colls.append((int(p[2]), int(p[3]), int(p[4]), int(p[5]), hx(p[6])))
            elif p[0] == "V":
                vir = [hx(v) for v in p[1:5]]
            elif p[0] == "T":
                tfin = (hx(p[1]), int(p[2]), int(p[3]))
            elif p[0] == "S":
                state.append([hx(v) for v in p[2:7]] + [int(p[7]), int(p[8])])
    init = np.array(init, dtype=object)
    state = np.array(state, dtype=object)
    c = np.array(colls, dtype=object) if colls else np.zeros((0, 5), dtype=object)
    return head, init, c, vir, tfin, state


def run_case(exe, args, maxcoll, trace, extra_env=None):
    env = dict(os.environ)
    env["MAXCOLL"] = str(maxcoll)
    env["TRACE_OUT"] = trace
    env.update(extra_env or {})
    subprocess.run([exe] + args.split(), env=env, check=True,
                   stdout=subprocess.DEVNULL)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("EDMD_REFERENCE_DIR"),
                    help="reference checkout (default: $EDMD_REFERENCE_DIR)")
    a = ap.parse_args()
    if not a.ref:
        ap.error("give --ref or set EDMD_REFERENCE_DIR to the reference checkout")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", "ref-additive", f"REF={a.ref}"],
                   check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_trace")
    exe_add = os.path.join(ROOT, "oracle", "_ref", "ref_trace_additive")
    tmp = os.path.join(HERE, "_tmp_trace.txt")
    cases = ([(n, c, exe, 0) for n, c in CASES.items()] + [(n, c, exe, 0) for n, c in TINY_CASES.items()]
             + [(n, c, exe, 0) for n, c in OPTION_CASES.items()]
             + [(n, c, exe_add, 1) for n, c in ADDITIVE_CASES.items()])
    for name, (args, maxcoll, full), case_exe, contact in cases:
        run_case(case_exe, args, maxcoll, tmp)
        head, init, c, vir, tfin, state = parse_trace(tmp)
        out = dict(
            args=np.array(args), contact=contact, N=head["N"], Lx=head["Lx"], Ly=head["Ly"],
            Nxc=head["Nxc"], Nyc=head["Nyc"],
            x0=init[:, 0].astype(np.float64), y0=init[:, 1].astype(np.float64),
            vx0=init[:, 2].astype(np.float64), vy0=init[:, 3].astype(np.float64),
            rad0=init[:, 4].astype(np.float64), m0=init[:, 5].astype(np.float64),
            type0=init[:, 6].astype(np.int32),
            ci=np.array([r[0] for r in c], np.int32),
            cj=np.array([r[1] for r in c], np.int32),
            ccell_i=np.array([r[2] for r in c], np.int32),
            ccell_j=np.array([r[3] for r in c], np.int32),
            ct=np.array([r[4] for r in c], np.float64),
            virial=np.array(vir, np.float64), t_final=tfin[0], ncol=tfin[1], ncross=tfin[2],
            xf=state[:, 0].astype(np.float64), yf=state[:, 1].astype(np.float64),
            cellf=state[:, 5].astype(np.int32), collf=state[:, 6].astype(np.int64),
        )
        if full:
            out.update(vxf=state[:, 2].astype(np.float64), vyf=state[:, 3].astype(np.float64),
                       radf=state[:, 4].astype(np.float64))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, "N", head["N"], "collisions", len(c), "t_final", tfin[0])
    for name, args in ABORT_CASES.items():
        env = dict(os.environ, MAXCOLL="1000000", TRACE_OUT=tmp)
        r = subprocess.run([exe] + args.split(), env=env, capture_output=True, text=True)
        assert r.returncode == 3, (name, r.returncode)
        m = re.search(r"between particle (\d+) and particle (\d+)", r.stdout + r.stderr)
        head, init, c, _, _, _ = parse_trace(tmp)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), args=np.array(args), contact=0,
                            N=head["N"], Lx=head["Lx"], Ly=head["Ly"], Nxc=head["Nxc"], Nyc=head["Nyc"],
                            x0=init[:, 0].astype(np.float64), y0=init[:, 1].astype(np.float64),
                            vx0=init[:, 2].astype(np.float64), vy0=init[:, 3].astype(np.float64),
                            rad0=init[:, 4].astype(np.float64), m0=init[:, 5].astype(np.float64),
                            type0=init[:, 6].astype(np.int32),
                            ci=np.array([x[0] for x in c], np.int32), cj=np.array([x[1] for x in c], np.int32),
                            ct=np.array([x[4] for x in c], np.float64),
                            pair=np.array([int(m.group(1)), int(m.group(2))], np.int32))
        print(name, "N", head["N"], "collisions before the abort", len(c), "pair", m.group(1), m.group(2))
    # verbatim dump + thermo files of a short run (ovito/LAMMPS text format pin)
    name, args = FILES_CASE
    dump = os.path.join(HERE, name + ".dump")
    thermo = os.path.join(HERE, name + ".thermo")
    run_case(exe, args, 10**12, tmp, {"DUMP_OUT": dump, "THERMO_OUT": thermo})
    head, init, c, vir, tfin, state = parse_trace(tmp)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), args=np.array(args), N=head["N"],
                        ncol=tfin[1], t_final=tfin[0])
    print(name, "N", head["N"], "collisions", len(c))
    for name, (args, contact) in FILES_GROW_CASES.items():
        dump = os.path.join(HERE, name + ".dump")
        thermo = os.path.join(HERE, name + ".thermo")
        run_case(exe_add if contact else exe, args, 10**12, tmp, {"DUMP_OUT": dump, "THERMO_OUT": thermo})
        h, _, cc, _, tf, _ = parse_trace(tmp)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), args=np.array(args), contact=contact,
                            N=h["N"], ncol=tf[1], t_final=tf[0])
        print(name, "N", h["N"], "collisions", len(cc))
    # the .txt restart state: "N Lx Ly", then "type x y rad m" per disk
    with open(os.path.join(HERE, LOAD_TXT), "w") as f:
        f.write("%d %.17g %.17g\n" % (head["N"], head["Lx"], head["Ly"]))
        for row in state:
            f.write("1 %.17g %.17g %.17g 1\n" % (row[0], row[1], row[4]))
    for name, args in LOAD_CASES.items():
        dump = os.path.join(HERE, name + ".dump")
        thermo = os.path.join(HERE, name + ".thermo")
        run_case(exe, args.format(golden=HERE), 10**12, tmp, {"DUMP_OUT": dump, "THERMO_OUT": thermo})
        head, init, c, vir, tfin, state = parse_trace(tmp)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), args=np.array(args), N=head["N"],
                            ncol=tfin[1], t_final=tfin[0],
                            x0=init[:, 0].astype(np.float64), y0=init[:, 1].astype(np.float64),
                            vx0=init[:, 2].astype(np.float64), vy0=init[:, 3].astype(np.float64),
                            xf=state[:, 0].astype(np.float64), yf=state[:, 1].astype(np.float64))
        print(name, "N", head["N"], "collisions", len(c))
    os.remove(tmp)


if __name__ == "__main__":
    sys.exit(main())
