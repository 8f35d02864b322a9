import numpy as np


class array:
    @staticmethod
    def from_euler_angles(alpha, beta, gamma):
        a, b, g = (np.atleast_1d(x) for x in (alpha, beta, gamma))
        return [(float(x), float(y), float(z)) for x, y, z in zip(a, b, g)]
