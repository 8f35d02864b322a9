import numpy as np


class Wigner:
    def __init__(self, J):
        self.J = J

    def Dindex(self, j, m, k):
        return (m + j) * (2 * j + 1) + (k + j)

    def D(self, angles):
        from richmol.rot.wig import wig_D
        a, b, g = angles
        d = wig_D(self.J, np.array([a]), np.array([b]), np.array([g]))[:, :, 0]
        return d.reshape(-1)
