"""Builds and runs the pipe-rate probe: `python -m psyclonebench_gb300.probes`."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    exe = os.path.join(HERE, "pipe_rates")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-fmad=false",
                    "-o", exe,
                    os.path.join(HERE, "pipe_rates.cu")], check=True)
    sys.exit(subprocess.run([exe]).returncode)


if __name__ == "__main__":
    main()
