"""Build and run oracle/opcount.cpp (algorithmic FP64 operation counts of
the oracle's restatement of the reference step).  Test infrastructure; the
numbers feed the roofline arithmetic in bench.py.

    python oracle/opcount.py [n] [cfl]          (reference formulation)
    python oracle/opcount.py --device [n]       (device formulation)
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(argv):
    os.makedirs(os.path.join(HERE, "_ref"), exist_ok=True)
    if argv and argv[0] == "--device":
        argv = argv[1:]
        exe = os.path.join(HERE, "_ref", "opcount_device")
        obj = os.path.join(HERE, "_ref", "gpr_oracle_count.o")
        subprocess.run(["gcc", "-O2", "-c", "-o", obj, os.path.join(HERE, "gpr_oracle.c")],
                       check=True)
        cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
        subprocess.run(["g++", "-O2", "-std=c++17", "-w", "-I" + cuda_inc, "-o", exe,
                        os.path.join(HERE, "opcount_device.cpp"), obj, "-lm"], check=True)
    else:
        exe = os.path.join(HERE, "_ref", "opcount")
        subprocess.run(["g++", "-O2", "-std=c++17", "-fpermissive", "-w", "-o", exe,
                        os.path.join(HERE, "opcount.cpp"), "-lm"], check=True)
    r = subprocess.run([exe] + argv, capture_output=True, text=True, check=True)
    sys.stdout.write(r.stdout)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
