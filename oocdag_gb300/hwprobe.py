"""Hardware facts the out-of-core schedule depends on, measured on the current GPU machine.

    python -m oocdag_gb300.hwprobe

Prints one JSON object: host RAM and cores (what bounds the host-resident matrix), the
FP64 DMMA rate (the plain path's roofline, from the library's probe) and page-locked
host<->device copy bandwidth (what bounds panel streaming), measured with CUDA events.
"""
from __future__ import annotations

import json
import os


def host_ram_bytes() -> int:
    with open("/proc/meminfo") as f:
        for line in f:
            if line.startswith("MemTotal:"):
                return int(line.split()[1]) * 1024
    return 0


def copy_bandwidth(nbytes: int = 4 << 30, reps: int = 3) -> dict:
    import torch

    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    h.fill_(1)
    s = torch.cuda.Stream()
    out = {}
    for name, (dst, src) in {"h2d_gbs": (d, h), "d2h_gbs": (h, d)}.items():
        best = 0.0
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(s):
                e0.record(s)
                dst.copy_(src, non_blocking=True)
                e1.record(s)
            torch.cuda.synchronize()
            best = max(best, nbytes / (e0.elapsed_time(e1) / 1e3) / 1e9)
        out[name] = best
    return out


def main() -> None:
    import torch

    import oocdag_gb300 as ooc

    props = torch.cuda.get_device_properties(0)
    with ooc.Handle(0) as h:
        fp64 = h.fp64_peak(300.0)
    res = {
        "gpu": props.name,
        "sms": props.multi_processor_count,
        "hbm_bytes": props.total_memory,
        "host_ram_bytes": host_ram_bytes(),
        "host_cores": os.cpu_count(),
        "fp64_dmma_tflops": fp64,
        **copy_bandwidth(),
    }
    print(json.dumps(res))


if __name__ == "__main__":
    main()
