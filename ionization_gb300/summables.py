"""``a + b`` composition for potentials, time windows, masks and states.

User code combines these objects with ``+`` (``CoulombPotential() +
SoftCoulombPotential()``, a superposition of states), the interface of
ionization/summables.py:6-80 (``Summand`` and ``Sum``).  Here a leaf is its
own only member; ``a + b`` makes an instance of ``a.summation_class`` whose
members are the members of ``a`` followed by those of ``b`` (composites
flatten, they never nest); calling a composite folds its members' values with
the composite's ``fold`` (addition unless a family says otherwise: masks and
time windows multiply).  Each composite family names the attribute its
members are read through (``container_name``: ``potentials``, ``masks``,
``states``, ...), which is made a read-only view of the member tuple.
"""

import operator
from functools import reduce


class Summand:
    """A leaf of a composition."""

    def __init__(self, *args, **kwargs):
        self.summation_class = Sum

    def members(self) -> tuple:
        return (self,)

    def __iter__(self):
        return iter(self.members())

    def __add__(self, other):
        return self.summation_class(*self.members(), *other)

    def __call__(self, *args, **kwargs):
        raise NotImplementedError

    def __str__(self):
        return type(self).__name__

    def __repr__(self):
        return self.__str__()


class Sum(Summand):
    """A composite: an ordered tuple of leaves."""

    container_name = "summands"
    fold = staticmethod(operator.add)

    def __init_subclass__(cls, **kwargs):
        super().__init_subclass__(**kwargs)
        name = cls.__dict__.get("container_name")
        if name:
            setattr(cls, name, property(Sum.members, doc="the members, in order"))

    def __init__(self, *members, **kwargs):
        self._members = tuple(members)
        super().__init__(**kwargs)

    def members(self) -> tuple:
        return self._members

    def __getitem__(self, index):
        return self._members[index]

    def __add__(self, other):
        # a composite keeps its own class whatever the other operand is
        return type(self)(*self._members, *other)

    def __call__(self, *args, **kwargs):
        return reduce(self.fold, (m(*args, **kwargs) for m in self._members))

    def __str__(self):
        return "(" + " + ".join(map(str, self._members)) + ")"

    def __repr__(self):
        return f"{type(self).__name__}({', '.join(map(repr, self._members))})"


Sum.summands = property(Sum.members, doc="the members, in order")
