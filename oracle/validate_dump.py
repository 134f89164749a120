"""rdp-validate-dump for this project (the reference's rdp_validate_dump.cpp): plays an RDPDUMP2
capture into the GPU path and into the CPU oracle side by side and compares TMEM, RDRAM and hidden
RDRAM after every draw (or every SyncFull with --sync-only).  Test infrastructure: the oracle is the
reference side.

    python oracle/validate_dump.py <dump> [--begin-frame N] [--sync-only] [--device D]

Exit status 0 when every comparison matched, 1 at the first difference (reported with its frame,
draw or sync number, address and pixel coordinate).
"""
import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [HERE, os.path.join(os.path.dirname(HERE), "parallel-rdp_gb300")]


class OracleTarget:
    """The CPU oracle as one side of the validation (it renders each command as it arrives)."""

    def __init__(self, rdram_size=8 << 20):
        from oracle import Oracle
        self.o = Oracle(rdram_size)

    def enqueue(self, words):
        self.o.enqueue(words)

    def idle(self):
        pass

    def rdram(self):
        return self.o.rdram()

    def hidden(self):
        return self.o.hidden()

    def tmem(self):
        return self.o.tmem()

    def write_rdram(self, data):
        self.o.write_rdram(data)

    def write_hidden(self, data):
        self.o.write_hidden(data)

    def close(self):
        self.o.close()


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("dump")
    ap.add_argument("--begin-frame", type=int, default=0)
    ap.add_argument("--sync-only", action="store_true")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    import numpy as np
    from rdp_gb300 import CommandProcessor
    from rdp_gb300.validate import GpuTarget, validate_dump
    ref = OracleTarget()
    with CommandProcessor(np.zeros(8 << 20, np.uint8), device=args.device) as cp:
        report = validate_dump(args.dump, ref, GpuTarget(cp), sync_only=args.sync_only, begin_frame=args.begin_frame)
    ref.close()
    print(json.dumps(report))
    return 0 if report["passed"] else 1


if __name__ == "__main__":
    sys.exit(main())
