"""Build and run oracle/opcount.cpp (algorithmic FP64 operation counts of
the oracle's restatement of the reference step).  Test infrastructure; the
numbers feed the roofline arithmetic in bench.py.

    python oracle/opcount.py [n] [cfl]
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(argv):
    exe = os.path.join(HERE, "_ref", "opcount")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-fpermissive", "-w", "-o", exe,
                    os.path.join(HERE, "opcount.cpp"), "-lm"], check=True)
    r = subprocess.run([exe] + argv, capture_output=True, text=True, check=True)
    sys.stdout.write(r.stdout)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
