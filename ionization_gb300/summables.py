"""Summand / Sum algebra used by potentials, masks and states.

Same behaviour as ionization/summables.py:6-80: ``a + b`` builds the
summation class of ``a`` from the members of both operands, calling a Sum
adds (or, for masks and windows, multiplies) its members' results.
"""


class Summand:
    def __init__(self, *args, **kwargs):
        self.summation_class = Sum

    def __str__(self):
        return self.__class__.__name__

    def __repr__(self):
        return str(self)

    def __iter__(self):
        yield self

    def __add__(self, other):
        return self.summation_class(*self, *other)

    def __call__(self, *args, **kwargs):
        raise NotImplementedError


class Sum(Summand):
    container_name = "summands"

    def __init__(self, *summands, **kwargs):
        setattr(self, self.container_name, summands)
        super().__init__(**kwargs)

    @property
    def _container(self):
        return getattr(self, self.container_name)

    def __str__(self):
        return "({})".format(" + ".join(str(s) for s in self._container))

    def __repr__(self):
        return "{}({})".format(self.__class__.__name__, ", ".join(repr(p) for p in self._container))

    def __iter__(self):
        yield from self._container

    def __getitem__(self, item):
        return self._container[item]

    def __add__(self, other):
        return self.__class__(*self, *other)

    def __call__(self, *args, **kwargs):
        return sum(x(*args, **kwargs) for x in self._container)
