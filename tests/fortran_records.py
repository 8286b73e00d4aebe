"""Independent reader of gfortran unformatted sequential files (test
infrastructure): each logical record is one or more subrecords, each framed
by signed 4-byte length markers; a negative leading marker means the record
continues in the next subrecord, a negative trailing marker that the
subrecord continues a previous one."""
import numpy as np


def read_records(path):
    data = open(path, "rb").read()
    out, pos, cur, first = [], 0, bytearray(), True
    while pos < len(data):
        lead = int(np.frombuffer(data, "<i4", 1, pos)[0])
        n = abs(lead)
        cur += data[pos + 4: pos + 4 + n]
        tail = int(np.frombuffer(data, "<i4", 1, pos + 4 + n)[0])
        assert abs(tail) == n, "trailing marker does not match"
        assert (tail < 0) == (not first), "continuation flag of the trailing marker"
        pos += 8 + n
        if lead < 0:
            first = False
        else:
            out.append(bytes(cur))
            cur, first = bytearray(), True
    assert not cur, "unterminated record"
    return out


def parse_fields(rec):
    """mx, my, mz, ex, ey, ez, bx, by, bz, dseed, lap, xinject, xinject2,
    xinject3, leftwall, walloc (code/output.F90:2200-2201)"""
    mx, my, mz = np.frombuffer(rec, "<i4", 3, 0)
    lot = int(mx) * int(my) * int(mz)
    f = np.frombuffer(rec, "<f4", 6 * lot, 12).reshape(6, lot)
    o = 12 + 24 * lot
    dseed = np.frombuffer(rec, "<f8", 1, o)[0]
    lap = np.frombuffer(rec, "<i4", 1, o + 8)[0]
    xinj = np.frombuffer(rec, "<f8", 3, o + 12)
    leftwall = np.frombuffer(rec, "<f4", 1, o + 36)[0]
    walloc = np.frombuffer(rec, "<f8", 1, o + 40)[0]
    assert len(rec) == o + 48
    return dict(dims=(int(mx), int(my), int(mz)), fields=dict(zip(("ex", "ey", "ez", "bx", "by", "bz"), f)),
                dseed=float(dseed), lap=int(lap), xinject=tuple(float(v) for v in xinj), leftwall=float(leftwall),
                walloc=float(walloc))


def parse_particles(rec, dtype):
    """ions, lecs, maxptl, maxhlf, totalpartnum, then each component for the
    ions and then the electrons (code/output.F90:2202-2218)"""
    ions, lecs, maxptl, maxhlf, total = (int(v) for v in np.frombuffer(rec, "<i4", 5, 0))
    pi = np.zeros(ions, dtype)
    pe = np.zeros(lecs, dtype)
    o = 20
    for name in ("x", "y", "z", "u", "v", "w", "ch", "ind", "proc", "splitlev"):
        t = "<f4" if name in ("x", "y", "z", "u", "v", "w", "ch") else "<i4"
        pi[name] = np.frombuffer(rec, t, ions, o)
        o += 4 * ions
        pe[name] = np.frombuffer(rec, t, lecs, o)
        o += 4 * lecs
    assert o == len(rec)
    return dict(ions=pi, lecs=pe, maxptl=maxptl, maxhlf=maxhlf, totalpartnum=total)
