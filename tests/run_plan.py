"""Run one batched plan on seeded device data a few times, for profiling.

    python tests/run_plan.py KIND DIMS BATCH [REPS] [FORM]
    python tests/run_plan.py queue COUNT [REPS]

The second form runs the first COUNT transforms of the mixed ("uneven")
batch as one queue (fft_gb300/uneven.py, seed 5) REPS times.

KIND is c, ci, r or ri; DIMS a JSON list such as [256,256,256]; FORM plain
(default), tc or f64 (double data through the FP64 kernels).  Each
repetition launches the plan's kernels once on the CUDA default stream;
the script synchronises at the end and prints the launches per transform.
"""
import json
import os
import sys

import torch

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from fft_gb300 import BatchPlan  # noqa: E402


def run_queue(count, reps):
    from fft_gb300 import Queue, uneven as U
    items = U.uneven_batch(10000, seed=5)[:count]
    buf, offs = U.allocate(items, torch.device("cuda"))
    q = Queue(U.descs(items, buf, offs))
    for _ in range(reps):
        q.run()
    torch.cuda.synchronize()
    print("queue of %d transforms, %d launches per run" % (count, q.launches))
    return 0


def main(argv):
    if len(argv) >= 2 and argv[0] == "queue":
        return run_queue(int(argv[1]), int(argv[2]) if len(argv) > 2 else 2)
    if len(argv) < 3:
        print(__doc__)
        return 2
    kind, dims, batch = argv[0], json.loads(argv[1]), int(argv[2])
    reps = int(argv[3]) if len(argv) > 3 else 2
    form = argv[4] if len(argv) > 4 else "plain"
    dt = torch.float64 if form == "f64" else torch.float32
    n = 1
    for d in dims:
        n *= d
    h = (dims[0] // 2 + 1) * (n // dims[0])
    plan = BatchPlan(kind, dims, batch, form=None if form == "plain" else form)
    g = torch.Generator(device="cuda").manual_seed(n + batch)
    nin = (h if kind == "ri" else n) * batch
    nout = (h if kind == "r" else n) * batch
    a = torch.randn(nin, device="cuda", generator=g, dtype=dt)
    b = torch.randn(nin, device="cuda", generator=g, dtype=dt)
    oa = torch.empty(nout, device="cuda", dtype=dt)
    ob = torch.empty_like(oa)
    for _ in range(reps):
        plan.launch(a, None if kind == "r" else b, oa, None if kind == "ri" else ob)
    torch.cuda.synchronize()
    print("launches per transform", plan.launches)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
