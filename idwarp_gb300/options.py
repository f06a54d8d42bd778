"""Options handling compatible with baseclasses.BaseSolver as USMesh uses it.

Default-option entries are ``[type, default]``; when ``default`` is a list the
option is a choice and its first element is the default (the convention of
idwarp/UnstructuredMesh.py:124-145).  Keys are case-insensitive.
"""
import copy
import pprint


class Error(Exception):
    """Raised for invalid use of the mesh API (baseclasses.utils.Error)."""

    def __init__(self, message):
        msg = "\n+" + "-" * 78 + "+\n| IDWarp (GB300) Error: "
        i = 23
        for word in str(message).split():
            if len(word) + i + 1 > 78:
                msg += " " * (78 - i) + "|\n| " + word + " "
                i = 1 + len(word) + 1
            else:
                msg += word + " "
                i += len(word) + 1
        msg += " " * (78 - i) + "|\n+" + "-" * 78 + "+\n"
        super().__init__(msg)


class BaseSolver:
    def __init__(self, name, category, defaultOptions=None, options=None, comm=None):
        self.name = name
        self.category = category
        self.comm = comm
        self._defaults = {}
        self._caseMap = {}
        self.options = {}
        for key, spec in (defaultOptions or {}).items():
            typ, default = spec
            low = key.lower()
            self._caseMap[low] = key
            if isinstance(default, list):
                self._defaults[low] = (typ, default[0], list(default))
            else:
                self._defaults[low] = (typ, default, None)
            self.options[low] = copy.deepcopy(self._defaults[low][1])
        for key, val in (options or {}).items():
            self.setOption(key, val)

    def _checkOption(self, key, val):
        low = key.lower()
        if low not in self._defaults:
            raise Error("Option '%s' is not a valid %s option." % (key, self.name))
        typ, _, choices = self._defaults[low]
        types = typ if isinstance(typ, tuple) else (typ,)
        if float in types and isinstance(val, int) and not isinstance(val, bool):
            val = float(val)
        if not isinstance(val, types):
            raise Error("Datatype for option '%s' was not valid. Expected %s, received %s." % (key, types, type(val)))
        if choices is not None and val not in choices:
            raise Error("Option '%s' must be one of %s, received %r." % (key, choices, val))
        return low, val

    def setOption(self, name, value):
        low, val = self._checkOption(name, value)
        self.options[low] = copy.deepcopy(val)

    def getOption(self, name):
        low = name.lower()
        if low not in self.options:
            raise Error("Option '%s' is not a valid %s option." % (name, self.name))
        return self.options[low]

    def printOptions(self):
        if self.comm is None or getattr(self.comm, "rank", 0) == 0:
            out = {self._caseMap[k]: v for k, v in self.options.items()}
            print("+" + "-" * 60 + "+")
            print("| %s options" % self.name)
            pprint.pprint(out)
            print("+" + "-" * 60 + "+")
