"""Times the reference's own host sky build (src/sky.cpp gendaymtx_step + src/solar.cpp sun_noaa, compiled unchanged by
`make -C oracle ref` where the reference tree is present) on the urban weather year, the work the precision benchmark's
GPU sky build does (bench.py urban_year_sky): a reported baseline, serial as the reference's run.cpp runs it.
Prints one JSON line. Baseline infrastructure only: nothing in the engine uses it."""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TOOL = os.path.join(HERE, "_ref", "ref_sky_golden")


def main(mf=4):
    subprocess.check_call(["make", "-s", "-C", HERE, "ref"])
    w = np.load(os.path.join(HERE, "..", "tests", "golden", "urban_sky", "weather.npy")).astype(np.float64)   # [2, 8760]
    with tempfile.TemporaryDirectory() as d:
        fi, fo = os.path.join(d, "w.bin"), os.path.join(d, "t.bin")
        np.ascontiguousarray(w.T).tofile(fi)
        subprocess.check_call([TOOL, "year", fi, fo, str(w.shape[1]), str(mf)])
        sec = float(np.fromfile(fo, np.float64)[0])
    print(json.dumps({"reference_host_sky_s": sec, "steps": int(w.shape[1]), "mf": mf, "patches": 144 * mf * mf + 1,
                      "threads": 1, "host": os.uname().machine}))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 4)
