"""BDF settings from option names, as the reference's bdf::options parses
them (time-integrators/bdf_parameters.hh:116-156, bdf_parameters.cc:6-105),
through the library's fs_bdf_settings_default (no device needed)."""
import math

import pytest

from flecsolve_gb300 import _lib
from flecsolve_gb300.time_integrator import bdf


def test_defaults_are_the_option_defaults():
    s = bdf.settings()
    # bdf_parameters.hh:126-155
    assert s.use_predictor == 1 and s.has_source_term == 0 and s.use_initial_predictor == 1
    assert s.dt_cut_lower_bound == 0.58754407 and s.dt_growth_upper_bound == 1.702
    assert s.number_of_time_intervals == 100
    assert s.use_pi_controller == 1 and s.pi_controller_type == 1  # PC.4.7
    assert s.control_timestep_variation == 0 and s.time_error_scaling == 1  # fixed-scaling
    assert s.time_rtol == 1e-9 and s.time_atol == 1e-15 and s.combine_timestep_estimators == 0
    # parameters.hh:35-42: max-dt, min-dt, initial-dt
    assert s.max_dt == 1.7976931348623157e308 and s.min_dt == 2.2250738585072014e-308
    assert s.initial_dt == 0.0
    # required options have no default
    assert math.isnan(s.initial_time) and math.isnan(s.final_time) and s.max_steps == -1
    assert s.integrator == -1 and s.starting_integrator == -1 and s.predictor == -1
    assert s.timestep_strategy == -1


def test_enum_parsers():
    # predictor and strategy are lower-cased before matching; methods,
    # controllers and error scalings are matched as written
    s = bdf.settings(predictor="LeapFrog", timestep_selection_strategy="Truncation-Error",
                     integrator="BDF3", starting_integrator="BE", pi_controller_type="H211b",
                     time_error_scaling="fixed-resolution", time_trunc_error_norm="l2")
    assert (s.predictor, s.timestep_strategy, s.integrator, s.starting_integrator) == (1, 0, 3, 1)
    assert (s.pi_controller_type, s.time_error_scaling, s.time_trunc_err_norm) == (0, 0, 1)
    for key, bad in (("integrator", "bdf3"), ("pi-controller-type", "pc11"), ("predictor", "euler"),
                     ("time-error-scaling", "Fixed-Scaling")):
        with pytest.raises(ValueError):
            bdf.settings(**{key: bad})


def test_option_names_and_values():
    s = bdf.settings(**{"initial-time": 0.5, "final-time": 2.0, "max-steps": 10, "initial-dt": 0.1,
                        "trunc-error-rtol": 1e-7, "trunc-error-atol": 1e-5, "problem-scales": [2.0],
                        "use-pi-controller": "false", "control-timestep-variation": "true"})
    assert (s.initial_time, s.final_time, s.max_steps, s.initial_dt) == (0.5, 2.0, 10, 0.1)
    assert (s.time_rtol, s.time_atol) == (1e-7, 1e-5)
    assert (s.num_problem_scales, s.problem_scale) == (1, 2.0)
    assert (s.use_pi_controller, s.control_timestep_variation) == (0, 1)
    with pytest.raises(ValueError):
        bdf.settings(problem_scales=[1.0, 2.0])  # one component
    with pytest.raises(KeyError):
        bdf.settings(no_such_option=1)


def test_enum_values_follow_the_reference_declaration_order():
    # bdf_parameters.hh:16-24
    assert [bdf.settings(integrator=m).integrator for m in ("CN", "BE", "BDF2", "BDF6")] == [0, 1, 2, 6]
    assert [bdf.settings(timestep_selection_strategy=t).timestep_strategy
            for t in ("truncation-error", "constant", "final-constant", "limit-relative-change")] == [0, 1, 2, 3]
    assert [bdf.settings(pi_controller_type=c).pi_controller_type
            for c in ("H211b", "PC.4.7", "PC11", "Deadbeat")] == [0, 1, 2, 3]
    assert _lib.BdfSettings is type(bdf.settings())
