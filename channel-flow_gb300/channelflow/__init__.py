"""GB300 (sm_103a) RK3-substep library for the staggered finite-difference
channel solver of Adrian-Lozano/channel-flow: Python host mirror of the
reference's time-integration interface over the C ABI of libchannel_gpu.so."""
from . import grids
from .lib import (ENS_TUNE_CANDIDATES, PREC_FP64, PREC_SPLIT, Channel, CfError, Ensemble, CfParams, default_params, header_functions, load,
                  read_input_parameters, read_snapshot, statistics_file_name, write_snapshot, write_statistics)

__all__ = ["grids", "Channel", "CfError", "Ensemble", "CfParams", "default_params", "header_functions", "load",
           "read_input_parameters", "read_snapshot", "write_snapshot", "write_statistics", "statistics_file_name", "PREC_FP64", "PREC_SPLIT",
           "ENS_TUNE_CANDIDATES"]
