"""Writer of LNFL's binary line file (TAPE3) in the layout CLBLM reads
(clblm_LineData.f90:52-161, RDLIN clblm_ODLAY.f90:2645-2700): Fortran
unformatted sequential records framed by 4-byte byte counts, the file header,
then per block of up to 250 lines a panel header (VMIN, VMAX, NREC, NWDS) and
the INPUT_BLOCK of 39*250 four-byte words.  The library reads such files with
clblm_tape3_read (capi.read_tape3)."""
import struct

import numpy as np

NLINEREC = 250
MXBRDMOL = 7
_BLOCK_WORDS = 39 * NLINEREC


def _record(f, payload):
    f.write(struct.pack("<i", len(payload)))
    f.write(payload)
    f.write(struct.pack("<i", len(payload)))


def _chars(s, n=8):
    return s.encode()[:n].ljust(n, b" ")


def write_tape3(path, lines, title="CLBLM GB300"):
    """Write a line list (capi_types.Lines, sorted by vnu) as TAPE3."""
    n = lines.n
    mols = np.unique(lines.mol % 100)
    hlinid = b"".join(_chars(x) for x in [title, "", "", "", "", "", "", "3.2", "", "I"])
    bmolid = b"".join(_chars("") for _ in range(64))
    molcnt = np.zeros(64, np.int32)
    sumstr = np.zeros(64, np.float32)
    for m in mols:
        sel = (lines.mol % 100) == m
        if 1 <= m <= 64:
            molcnt[m - 1] = int(sel.sum())
            sumstr[m - 1] = float(lines.sp[sel].astype(np.float64).sum())
    zeros = np.zeros(64, np.int32)
    nblocks = (n + NLINEREC - 1) // NLINEREC
    key = lines.keys()  # the line centres; a coupling-coefficient record takes its line's
    header = (hlinid + bmolid + molcnt.tobytes() + zeros.tobytes() + zeros.tobytes() + sumstr.tobytes()
              + struct.pack("<i", len(mols)) + struct.pack("<ff", float(key[0]), float(key[-1]))
              + struct.pack("<iiiii", n, 0, 0, nblocks, nblocks) + _chars("") + _chars(""))
    with open(path, "wb") as f:
        _record(f, header)
        for b in range(nblocks):
            lo, hi = b * NLINEREC, min(n, (b + 1) * NLINEREC)
            k = hi - lo

            def pad(a, dt):
                out = np.zeros(NLINEREC, dt)
                out[:k] = a[lo:hi]
                return out.tobytes()
            body = (pad(lines.vnu, "<f8") + pad(lines.sp, "<f4") + pad(lines.alfa, "<f4") + pad(lines.epp, "<f4")
                    + pad(lines.mol, "<i4") + pad(lines.hwhm, "<f4") + pad(lines.tmpalf, "<f4")
                    + pad(lines.pshift, "<f4") + pad(lines.iflg, "<i4")
                    + np.zeros(MXBRDMOL * NLINEREC, "<i4").tobytes()
                    + np.zeros(3 * MXBRDMOL * NLINEREC, "<f4").tobytes()
                    + np.zeros(NLINEREC, "<f4").tobytes())
            assert len(body) == 4 * _BLOCK_WORDS  # 39*250 words, VNU two per line
            _record(f, struct.pack("<ddii", float(key[lo]), float(key[hi - 1]), k, len(body) // 4))
            _record(f, body)
