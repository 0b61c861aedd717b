"""GB300-native N-Queens constellation engine (sm_103a CUDA behind a C ABI).

Drop-in for the constellation solver of suzukiiichiro/N-Queens
(14Bit_codon_GPU/356Py_savesp_narrow.py): ``gen_constellations`` and
``exec_solutions`` keep the reference's signatures; ``Engine`` adds array
calls, batches and completion queries.
"""
from ._lib import NQError, RECORD_DTYPE, lib  # noqa: F401
from .engine import (Batch, CompletionJob, CountJob, Engine, Result, count, default_engine,  # noqa: F401
                     exec_solutions, gen_constellations, gen_records, gen_records_starts, gen_records_wide,
                     records_from_constellations, select_dynamic_preset_queens, start_constellations)

__all__ = ["Batch", "CompletionJob", "CountJob", "Engine", "NQError", "RECORD_DTYPE", "Result", "count",
           "default_engine", "exec_solutions", "gen_constellations", "gen_records", "gen_records_starts",
           "gen_records_wide", "records_from_constellations", "select_dynamic_preset_queens", "start_constellations",
           "lib"]
