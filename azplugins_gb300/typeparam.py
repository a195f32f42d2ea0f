"""Per-type parameter dictionaries with the key conventions of HOOMD's
``TypeParameterDict`` as azplugins uses them (``src/pair.py``, ``src/bond.py``):

* pair parameters are keyed by an unordered pair of type names, ``("A", "B")``
  and ``("B", "A")`` being the same entry (``len_keys=2``);
* bond parameters are keyed by a bond type name such as ``"A-A"``;
* a key may also be a list of names / pairs, which sets every one of them.
"""

from __future__ import annotations

import copy


class _Entry(dict):
    """The dict ``params[key]`` returns: a copy whose ``update`` / item assignment
    write back into the owner (``barrier.params["A"].update(k=..., offset=...)``
    as in src/pytest/test_external.py:65). Keys still missing stay missing until
    they are set; the tables that use the entry report them."""

    def __init__(self, owner, key, values):
        super().__init__(values)
        self._owner = owner
        self._key = key

    def _store(self):
        self._owner._data[self._key] = dict(self)

    def update(self, *args, **kw):
        new = dict(*args, **kw)
        self._owner._check_keys(new)
        super().update({k: float(v) for k, v in new.items()})
        self._store()

    def __setitem__(self, k, v):
        self._owner._check_keys({k: v})
        super().__setitem__(k, float(v))
        self._store()


class TypeParameterDict:
    """Dict of parameter dicts (or scalars) with required keys and defaults."""

    def __init__(self, len_keys: int, required=(), defaults=None, scalar=False, name="params"):
        self._len = len_keys
        self._required = tuple(required)
        self._defaults = dict(defaults or {})
        self._scalar = scalar
        self._name = name
        self._data = {}
        self._default_value = None

    # ------------------------------------------------------------------ keys
    def _norm(self, key):
        if self._len == 2:
            if not (isinstance(key, tuple) and len(key) == 2 and all(isinstance(k, str) for k in key)):
                raise KeyError(f"{self._name} keys are (type_a, type_b) tuples, got {key!r}")
            return tuple(sorted(key))
        if not isinstance(key, str):
            raise KeyError(f"{self._name} keys are type names, got {key!r}")
        return key

    def _expand(self, key):
        if isinstance(key, list):
            return [self._norm(k) for k in key]
        return [self._norm(key)]

    # ------------------------------------------------------------------ values
    def _check_keys(self, value):
        allowed = set(self._required) | set(self._defaults)
        extra = set(value) - allowed
        if extra:
            raise KeyError(f"{self._name}: unknown keys {sorted(extra)}; expected {sorted(allowed)}")

    def _validate(self, value):
        if self._scalar:
            return float(value)
        if not isinstance(value, dict):
            raise TypeError(f"{self._name} values are dicts, got {type(value).__name__}")
        self._check_keys(value)
        out = dict(self._defaults)
        out.update({k: float(v) for k, v in value.items()})
        missing = [k for k in self._required if k not in out]
        if missing:
            raise KeyError(f"{self._name}: missing required keys {missing}")
        return out

    def __setitem__(self, key, value):
        v = self._validate(value)
        for k in self._expand(key):
            self._data[k] = copy.copy(v)

    def __getitem__(self, key):
        k = self._norm(key)
        if self._scalar:
            if k in self._data:
                return self._data[k]
            if self._default_value is not None:
                return self._default_value
            raise KeyError(f"{self._name}[{key!r}] is not set")
        if k in self._data:
            return _Entry(self, k, self._data[k])
        if self._default_value is not None:
            return _Entry(self, k, self._default_value)
        if self._len == 1:
            # unset type: an entry holding the defaults, filled in by update()
            return _Entry(self, k, self._defaults)
        raise KeyError(f"{self._name}[{key!r}] is not set")

    def __contains__(self, key):
        try:
            k = self._norm(key)
        except KeyError:
            return False
        return k in self._data or self._default_value is not None

    def set_default(self, value):
        self._default_value = self._validate(value) if value is not None else None

    @property
    def default(self):
        return self._default_value

    def keys(self):
        return self._data.keys()

    def items(self):
        return self._data.items()

    def to_base(self):
        return {k: copy.copy(v) for k, v in self._data.items()}
