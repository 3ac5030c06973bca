"""Times the tcgen05 Ozaki engine's launch-shape knobs on one device-resident launch.

    python tiled-mm_gb300/peaks/engine_knobs.py '{}' '{"TMM_TC_PACE": 1}' '{"TMM_TC_GROUP_M": 8}'

Each argument is a JSON object of environment settings read by the engine at launch
(TMM_TC_PACE, TMM_TC_PACE_CHUNK, TMM_TC_PACE_NS, TMM_TC_GROUP_M, TMM_TC_PAIR_STAGES,
TMM_TC_CLUSTER); '{}' is the default form.  Per setting: one warm-up launch, then
KNOBS_REPS event-timed launches (ms), the median SM clock sampled during them, ms x GHz
(the launch in units of 10^6 cycles at that clock), the device status, and whether C is
bit-identical to the first setting's.  The launch is m = n = KNOBS_MN (32768), k = KNOBS_K
(16384), 11 slices, u*2^e entries with e in [-20, 20]."""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "tiled-mm_gb300"))
sys.path.insert(0, str(ROOT))

KEYS = ("TMM_TC_PACE", "TMM_TC_PACE_CHUNK", "TMM_TC_PACE_NS", "TMM_TC_GROUP_M", "TMM_TC_PAIR_STAGES", "TMM_TC_CLUSTER")


def main() -> None:
    import torch

    import bench
    import tiledmm as tmm

    m = n = int(os.environ.get("KNOBS_MN", "32768"))
    k = int(os.environ.get("KNOBS_K", "16384"))
    reps = int(os.environ.get("KNOBS_REPS", "3"))
    a = torch.empty(m * k, dtype=torch.float64, device="cuda")
    b = torch.empty(k * n, dtype=torch.float64, device="cuda")
    c = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    tmm.fill_device(a.data_ptr(), m, k, m, 2, 20.0, seed=0, mat_id=0)
    tmm.fill_device(b.data_ptr(), k, n, k, 2, 20.0, seed=0, mat_id=1)
    ctx = tmm.make_context(np.float64, 2, m, n, k)
    ctx.set_path(tmm.PATH_OZAKI, 11)
    sid = torch.cuda.current_stream().cuda_stream
    ref = None
    for arg in sys.argv[1:] or ["{}"]:
        cfg = json.loads(arg)
        for key in KEYS:
            os.environ.pop(key, None)
        os.environ.update({key: str(v) for key, v in cfg.items()})
        tmm.gemm_device(ctx, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m, stream=sid)
        torch.cuda.synchronize()
        times = []
        with bench.ClockSampler(0) as clk:
            for _ in range(reps):
                ctx.set_kernel_timing(True)
                tmm.gemm_device(ctx, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m, stream=sid)
                torch.cuda.synchronize()
                sec, _ = ctx.kernel_time()
                ctx.set_kernel_timing(False)
                times.append(sec * 1e3)
        status = ctx.device_status(sid)
        same = None
        if ref is None:
            ref = c.clone()
        else:
            same = bool(torch.equal(ref, c))
        cs = clk.summary()
        ms = float(np.median(times))
        mhz = cs.get("sm_mhz") or 0.0
        print(json.dumps({"cfg": cfg, "ms": [round(t, 1) for t in times], "ms_median": round(ms, 1), "sm_mhz": mhz,
                          "ms_x_ghz": round(ms * mhz / 1000, 1), "reasons": cs.get("reasons"), "status": status,
                          "identical": same}), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()
