"""PETSc binary vectors, the reference's file format for walls, ICs and fi.

IOView/IOLoad (lbm_io.F90:71-134) write VecView output: big-endian int32
class id 1211214, int32 length, then that many big-endian float64 in natural
order (dof fastest, then x, y, z).  A ``.info`` file carries the block size.
File names are ``<prefix><name><counter:03d>.dat``.
"""
import os

import numpy as np

VEC_CLASSID = 1211214


def write_vec(path, values, block_size=None):
    a = np.ascontiguousarray(values, dtype=np.float64).ravel()
    with open(path, "wb") as f:
        f.write(np.array([VEC_CLASSID, a.size], dtype=">i4").tobytes())
        f.write(a.astype(">f8").tobytes())
    if block_size is not None and block_size > 1:
        with open(path + ".info", "w") as f:
            f.write("-vecload_block_size %d\n" % block_size)


def read_vec(path):
    with open(path, "rb") as f:
        head = np.frombuffer(f.read(8), dtype=">i4")
        if head.size != 2 or head[0] != VEC_CLASSID:
            raise ValueError("%s: not a PETSc binary vector" % path)
        n = int(head[1])
        data = np.frombuffer(f.read(8 * n), dtype=">f8")
        if data.size != n:
            raise ValueError("%s: truncated (%d of %d values)" % (path, data.size, n))
    return data.astype(np.float64)


def output_name(prefix, name, counter):
    return "%s%s%03d.dat" % (prefix, name, counter)


def read_field(path, nsites, dof):
    a = read_vec(path)
    if a.size != nsites * dof:
        raise ValueError("%s: %d values, expected %d x %d" % (path, a.size, nsites, dof))
    return a


def exists(prefix, name, counter):
    return os.path.exists(output_name(prefix, name, counter))
