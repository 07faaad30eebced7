"""Result containers with the same interface as PyPO's (reference
src/PyPO/PyPOTypes.py:7-260): `currents` (Jx..Mz), `fields` (Ex..Hz),
`scalarfield` (S), `rfield` (x, y, z). Members are 2-D complex arrays shaped
like the target grid; `memlist` names them in bundle order; `setMeta` records
the surface name and wavenumber.
"""
import numpy as np


class resContainer:
    def __init__(self, *args, restype="EH"):
        self.type = restype
        self.memlist = []
        self.shape = np.shape(args[0])
        self.size = int(np.prod(self.shape))
        for i, arg in enumerate(args):
            name = f"{restype[i // 3]}{'xyz'[i % 3]}"
            self.memlist.append(name)
            setattr(self, name, arg)

    def setMeta(self, surf, k):
        self.surf = surf
        self.k = k

    def __getitem__(self, idx):
        try:
            return getattr(self, self.memlist[idx])
        except (IndexError, TypeError):
            raise IndexError(f"Index out of range: {idx}")

    def __setitem__(self, idx, item):
        try:
            setattr(self, self.memlist[idx], item)
        except (IndexError, TypeError):
            raise IndexError(f"Index out of range: {idx}")

    def T(self):
        for i in range(6):
            self[i] = self[i].T
        return self

    def H(self):
        for i in range(6):
            self[i] = self[i].conj().T
        return self

    def stack(self):
        """(6, *shape) complex array in memlist order."""
        return np.stack([self[i] for i in range(6)])


class currents(resContainer):
    def __init__(self, Jx, Jy, Jz, Mx, My, Mz):
        super().__init__(Jx, Jy, Jz, Mx, My, Mz, restype="JM")


class fields(resContainer):
    def __init__(self, Ex, Ey, Ez, Hx, Hy, Hz):
        super().__init__(Ex, Ey, Ez, Hx, Hy, Hz, restype="EH")


class rfield:
    def __init__(self, Prx, Pry, Prz):
        self.x = Prx
        self.y = Pry
        self.z = Prz
        self.shape = np.shape(Prx)


class scalarfield:
    def __init__(self, S):
        self.S = S

    def setMeta(self, surf, k):
        self.surf = surf
        self.k = k
