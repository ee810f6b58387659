"""Writes oracle/data/config2_image<i>.npz: the benchmark's config-2 pore images
(mantiis_gb300.workloads.config2: 1024x1024 seeded disks, radii U[6,40],
porosity U[0.5,0.7], mean Kn U[0.01,1]) as packed bits with the drawn mean Kn,
so that the CPU arm of bench.py (the oracle) rebuilds the same workload with
its own pore-property and grid code and loads no product library.

Test-infrastructure input; run once:  python oracle/make_inputs.py [count]
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def main(count=1):
    from mantiis_gb300 import workloads

    out = ROOT / "oracle" / "data"
    out.mkdir(exist_ok=True)
    for i in range(count):
        img = workloads.config2(i)
        pore = img["pore"].astype(np.uint8)
        n = pore.shape[0]
        np.savez_compressed(out / f"config2_image{i}.npz", pore_bits=np.packbits(pore.reshape(-1)), n=n,
                            kn_mean=img["kn_mean"], dx=img["dx"], levels=3, edge_fine=1)
        print(f"config2_image{i}: n {n}, porosity {img['porosity']:.4f}, mean Kn {img['kn_mean']:.6f}")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 1)
