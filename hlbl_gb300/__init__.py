"""hlbl_gb300: the connected HLbL kernel sum of jing2li/hlbl on one GB300.

Host side over the C ABI of libhlbl_gb300.so (include/hlbl_gb300.h). The
Contractor mirrors hlbl::Contractor (include/hlbl/contract.hpp of the
reference); the schedule helpers mirror src/schedule.cpp.

The native library is loaded on first use of a name that needs it; if it is
missing, that raises ImportError (there is no fallback).
"""
from importlib import import_module

_LAZY = {"Contractor": "contract", "FP64": "contract", "FP32": "contract", "xunit": "contract",
         "HlblError": "_lib", "QED_STANDIN": "contract", "QED_STANDIN_GENERIC": "contract",
         "QED_DENSE": "contract", "QED_DENSE_KERV": "contract", "QED_KQED": "contract"}

__all__ = ["Contractor", "FP64", "FP32", "xunit", "HlblError", "schedule", "QED_STANDIN",
           "QED_STANDIN_GENERIC", "QED_DENSE", "QED_DENSE_KERV", "QED_KQED"]


def __getattr__(name):
    if name in _LAZY:
        return getattr(import_module(f".{_LAZY[name]}", __name__), name)
    if name == "schedule":
        return import_module(".schedule", __name__)
    raise AttributeError(name)
