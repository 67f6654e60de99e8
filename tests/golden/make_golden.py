"""Generate the golden fixtures in this folder by running the reference's
own CPU code (oracle/_ref, built from the reference tree by oracle/Makefile).

  python tests/golden/make_golden.py

golden_fd2d_cpu.npz   CPU_vti2dfd (2D-3D-vti-fd-cuda-gtk-GUI/CPU_vti2dfd_kernels.c:366)
                      on a 61x51 layered VTI model, 250 steps, SV taper on
golden_rtm2d_mpi.npz  the MPI RTM (2D-vti-fd+rtm-mpi/Toa_rtm_vti_adcig_cdp.c,
                      model_vti_get_boundry + RTM_corr_adcig) for two shots with
                      different odd aperture widths, stacked, then laplac2_lop
                      (utils-Laplacian-filter/laplace.c) with adj=1
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import orc  # noqa: E402
from tests.util import layered_model  # noqa: E402


def main():
    orc.build(with_ref=True)
    v, e, d = layered_model(61, 51, seed=1)
    ref, _ = orc.ref_cpu_vti2dfd(v, e, d, npd=20, nt=250, dx=10, dz=10, dt_us=1000, favg=20, fs=30, zs=5, sv=1)
    np.savez_compressed(os.path.join(HERE, "golden_fd2d_cpu.npz"), v=v, e=e, d=d, shot=ref[0], npd=20, nt=250,
                        fs=30, zs=5, sv=1)
    rng = np.random.default_rng(3)
    nx, nz = 101, 50
    v, e, d = layered_model(nx, nz, seed=3, vlo=2000, vhi=2600)
    v += rng.uniform(0, 40, v.shape).astype(np.float32)
    acc = np.zeros((nx, nz), np.float32)
    shots, widths = [1, 2], [41, 53]
    for is_, nxs in zip(shots, widths):
        orc.ref_rtm_mpi_shot(v, e, d, acc, npd=15, nt=650, dx=10.0, dz=10.0, dt_ms=1.0, favg=20.0, pfac=1000.0,
                             fs_sxd=35, ds_sxd=20, zs_sxd=1, is_=is_, nxs=nxs)
    img = orc.ref_laplace2d_adj(acc)
    np.savez_compressed(os.path.join(HERE, "golden_rtm2d_mpi.npz"), v=v, e=e, d=d, image=img, stack=acc,
                        npd=15, nt=650, fs=35, ds=20, shots=shots, widths=widths)
    with open(os.path.join(HERE, "SHA256SUMS"), "w") as f:
        for name in sorted(os.listdir(HERE)):
            if name.endswith(".npz"):
                h = hashlib.sha256(open(os.path.join(HERE, name), "rb").read()).hexdigest()
                f.write("%s  %s\n" % (h, name))


if __name__ == "__main__":
    main()
