"""Empty h5py stand-in: jqmc/hamiltonians.py imports h5py at module level."""


class Group:
    pass


class Dataset:
    pass


class File:
    def __init__(self, *a, **k):
        raise NotImplementedError("HDF5 is not available")
