"""Stand-in for torchio: only the names the reference imports. File loading is
not used when generating fixtures (subjects are built from tensors)."""


class ScalarImage:  # pragma: no cover - never constructed
    def __init__(self, *a, **k):
        raise RuntimeError("torchio is not available")


class LabelMap(ScalarImage):  # pragma: no cover
    pass
