"""pytest plugin (test infrastructure): installs the oracle as ``miepy.cpp`` and
imports the reference package before the reference's own test modules load."""

from .refshim import import_reference

import_reference()
