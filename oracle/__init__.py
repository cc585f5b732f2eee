"""ORACLE — test infrastructure only: the CPU restatement of micrographia's engine semantics
(oracle.hpp) and its bindings (oracle.py). Only the tests, __graft_entry__.smoke() and bench.py's
CPU baseline use it, as the checker; the engine never does."""
