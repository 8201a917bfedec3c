"""Writes tests/golden/mtckd_h2o_0_3000.npz: the 0-3000 cm-1 slice of the
MT_CKD H2O continuum table that CLBLM ships
(clblm_data/spectroscopy/absco-ref_wv-mt-ckd.nc, read by
mt_ckd_h2o_module.f90:94-103: self_absco_ref, for_absco_ref, self_texp,
ref_press, ref_temp on a 10 cm-1 grid).

Usage: python tests/golden/make_mtckd_fixture.py <path of the CLBLM project>
"""
import sys
from pathlib import Path

import numpy as np
from scipy.io import netcdf_file

V_LO, V_HI = 0.0, 3000.0


def main(root):
    nc = Path(root) / "clblm_data" / "spectroscopy" / "absco-ref_wv-mt-ckd.nc"
    f = netcdf_file(str(nc), "r", mmap=False)
    wv = np.array(f.variables["wavenumbers"].data, dtype=np.float64)
    sel = (wv >= V_LO) & (wv <= V_HI)
    out = Path(__file__).resolve().parent / "mtckd_h2o_0_3000.npz"
    np.savez_compressed(out, wavenumbers=wv[sel],
                        self_absco_ref=np.array(f.variables["self_absco_ref"].data, dtype=np.float64)[sel],
                        for_absco_ref=np.array(f.variables["for_absco_ref"].data, dtype=np.float64)[sel],
                        self_texp=np.array(f.variables["self_texp"].data, dtype=np.float64)[sel],
                        ref_press=float(f.variables["ref_press"].data),
                        ref_temp=float(f.variables["ref_temp"].data))
    f.close()
    print(out, int(sel.sum()), "points")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else ".")
