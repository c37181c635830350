"""Load the committed golden fixtures (tests/golden/*.npz, made by running
the reference itself: tests/golden/make_golden.py) as test cases."""
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    d = np.load(os.path.join(HERE, name + ".npz"))
    case = dict(nx=int(d["nx"]), ny=int(d["ny"]), L=float(d["L"]), dt=float(d["dt"]),
                B=tuple(float(b) for b in d["B"]), species=[])
    for i in range(int(d["nspecies"])):
        case["species"].append(dict(q=float(d["q%d" % i]), m=float(d["m%d" % i]),
                                    x=d["x%d" % i], y=d["y%d" % i], ux=d["ux%d" % i], uy=d["uy%d" % i]))
    return case, d


def harmonic_case():
    return dict(nx=1024, ny=1024, L=8.0, dt=5e-3, B=(0.0, 0.0, 0.0),
                species=[dict(q=-1.0, m=1e-2, x=np.array([1.0]), y=np.array([4.0]),
                              ux=np.zeros(1), uy=np.zeros(1)),
                         dict(q=-1.0, m=1e-2, x=np.array([7.0]), y=np.array([4.0]),
                              ux=np.zeros(1), uy=np.zeros(1))])


def harmonic_trace():
    d = np.load(os.path.join(HERE, "harmonic.npz"))
    return d["x0"], d["Ex0"]
