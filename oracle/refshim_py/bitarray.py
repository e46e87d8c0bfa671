"""Test-only stand-in for the `bitarray` package, which the reference's
indexutils module imports at load time.  Enough of it for findMismatches
(construct with a length, setall, item assignment); the golden-vector
script reads the result back as a list of bits."""


class bitarray(list):  # noqa: N801 - name of the package's class
    def __init__(self, n=0):
        super().__init__([False] * (n if isinstance(n, int) else 0))

    def setall(self, v):
        for i in range(len(self)):
            self[i] = bool(v)
