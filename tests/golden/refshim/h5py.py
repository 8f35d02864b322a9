def is_hdf5(filename):
    return False
