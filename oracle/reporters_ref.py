"""ORACLE — TEST INFRASTRUCTURE ONLY.

Python restatement of the record layouts of fortran/reporters.f90, used by
the tests to check the library's reporters byte for byte from the same
(FP32, promoted) state. Edit descriptors: F0.d = shortest fixed form with d
decimals and a leading zero; I0 = shortest integer; list-directed integers
right-justified in 12 columns; nX after the last item of a record writes
nothing; an empty list-directed WRITE is an empty line.
"""
import numpy as np


def F(x, d):
    return f"{float(x):.{d}f}"


def rec(items, lead=False):
    return (" " if lead else "") + "  ".join(items) + "\n"


def lst(i):
    return f"{int(i):12d}\n"


def body_z(q):
    w, x, y, z = q
    return 2.0 * (x * z + w * y), 2.0 * (y * z - w * x), w * w - x * x - y * y + z * z


def state_header():   # open_state_data_file (reporters.f90:7-19)
    return "Step  Potential_Energy  Kinetic_Energy  Total_Energy  Temperature  Pressure  Density\n"


def state_line(step, n, pot, kin, rot, temp, pres, dens):   # report_state_data (:21-37)
    pa, ka, ra = pot / n, kin / n, rot / n
    return rec([str(step)] + [F(v, 10) for v in (pa, ka + ra, pa + ka + ra, temp, pres, dens)])


def trajectory(step, box, types, shape, r, q, f):   # report_trajectory (:66-92)
    out = "ITEM: TIMESTEP\n" + lst(step) + "ITEM: NUMBER OF ATOMS\n" + lst(len(r)) + "ITEM: BOX BOUNDS pp pp pp\n"
    for d in range(3):
        out += rec([F(-box[d] / 2.0, 3), F(box[d] / 2.0, 3)], lead=True)
    out += "ITEM: ATOMS id type shapex shapey shapez x y z vx vy vz fx fy fz quatw quati quatj quatk\n"
    for i in range(len(r)):
        u = body_z(q[i])
        vals = list(shape[i]) + list(r[i]) + list(u) + list(f[i]) + list(q[i])
        out += rec([str(i + 1), str(types[i])] + [F(v, 3) for v in vals], lead=True)
    return out


def config(r, v, l, q):   # report_confwriter (:120-129)
    return "".join(rec([F(x, 3) for x in list(r[i]) + list(v[i]) + list(l[i]) + list(q[i])]) for i in range(len(r)))


def checkpoint(box, types, mass, charge, sig, eps, inertia, r, v, l, q, bonds, config_index=0):   # (:158-184)
    n = len(r)
    out = f"ATOMS {n}\n\nBONDS {len(bonds)}\n\nBOX " + rec([F(b, 10) for b in box])
    out += ("\nATOM: ID TYPE MASS CHARGE SHAPEX SHAPEY SHAPEZ ESHAPEX ESHAPEY ESHAPEZ IXX IYY IZZ RX RY RZ VX VY VZ "
            "LX LY LZ QW QX QY QZ\n\n")
    for i in range(n):
        vals = [mass[i], charge[i]] + list(sig[i]) + list(eps[i]) + list(inertia[i]) + list(r[i]) + list(v[i]) + \
            list(l[i]) + list(q[i])
        out += rec([str(i + 1), str(types[i])] + [F(x, 10) for x in vals], lead=True)
    out += "\nBOND: ID I J LEN\n\n"
    for k, (i, j, ln) in enumerate(bonds):
        out += rec([str(k + 1), str(i + 1), str(j + 1), F(ln, 10)], lead=True)
    return out + "\n" + lst(config_index)
