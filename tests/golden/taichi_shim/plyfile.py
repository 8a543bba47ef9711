"""Stand-in for ``plyfile`` (absent here); the golden scenes use no PLY input."""


class PlyData:  # pragma: no cover - never used by the golden scenes
    @staticmethod
    def read(path):
        raise RuntimeError("plyfile stand-in: PLY input is not supported by the golden generator")


class PlyElement:  # pragma: no cover
    @staticmethod
    def describe(*a, **k):
        raise RuntimeError("plyfile stand-in: PLY output is not supported by the golden generator")
