def lebedev(*args):
    raise NotImplementedError("Lebedev quadrature is not available in this environment")


def lebedev_npoints(*args):
    raise NotImplementedError("Lebedev quadrature is not available in this environment")
