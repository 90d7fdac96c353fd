"""Stand-in exposing the names the reference imports; any use raises."""


class _Unavailable:
    def __init__(self, *a, **k):
        raise RuntimeError("h5py is not installed; the golden generator keeps all data in memory")


class File(_Unavailable):
    pass


class Group(_Unavailable):
    pass


class Dataset(_Unavailable):
    pass
