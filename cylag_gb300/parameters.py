"""Solver parameters: the reference's dict of options, checked the same way.

Mirrors ``cylag.Parameters`` (cylag/core/parameters.pyx:116-351) and the
defaults of ``CYLAG_DEFAULT_PARAMETERS`` (cylag/cylag_dico.py:9-51):

* keys absent from the defaults, or values whose type differs from the
  default's, raise ``TypeError`` (parameters.pyx:318-351);
* ``time_scheme``, when not given, follows model and diffusion
  (parameters.pyx:179-195);
* out-of-range values raise ``ValueError`` (parameters.pyx:197-316).

Two keys exist only here and are not part of the reference dict; they are
passed separately to ``Solver`` (``precision=`` and ``sort_period=``).
"""
from __future__ import annotations

CYLAG_DEFAULT_PARAMETERS = {
    "initial_time": 0.,
    "final_time": 3600.,
    "time_step": 1.,
    "frozen_eulerian_fields": False,
    "model": 1,
    "time_scheme": 1,
    "particle_velocity_init": 1,
    "rng_method": 2,
    "lsm3_edge_opt": 2,
    "water_density": 1000.,
    "diffusion_model": 0,
    "horizontal_diffusivity": 0.,
    "vertical_diffusivity": 0.,
    "schmidt_number": 0.72,
    "diffusion_lsm2_option": 1,
    "diffusion_lsm3_tl_horizontal": 1.,
    "diffusion_lsm3_tl_vertical": 1.,
    "boundary_conditions": True,
    "boundary_conditions_type": 1,
    "boundary_conditions_debug": False,
    "max_wall_rebounds": 4,
    "rebound_damping_coef": 0.5,
    "wall_roughness_angle": 15.0,
    "stranding_probability": 0.,
    "listing": False,
    "listing_printout_period": 10,
    "output_rep": "particles",
    "output_file": False,
    "output_printout_period": 10,
    "output_file_format": "txt",
    "output_file_name": "particles",
    "bnd_statistics": False,
    "bnd_statistics_file_name": "bnd_stats",
    "control_sections_file_name": "cs_stats",
    "stranding_output": False,
    "stranding_output_file_name": "stranded_particles",
}


class Parameters:
    """Attribute view of the merged parameter dict."""

    def __init__(self, parameters=None):
        parameters = {} if parameters is None else dict(parameters)
        params = dict(CYLAG_DEFAULT_PARAMETERS)
        params.update(parameters)
        self.check_types(CYLAG_DEFAULT_PARAMETERS, params)
        for k, v in params.items():
            setattr(self, k, v)
        if self.frozen_eulerian_fields:
            self.initial_time = 0.
        self.control_sections = False
        self.ncsec = 0
        if "time_scheme" not in parameters:
            if self.model == 1 and self.diffusion_model == 0:
                self.time_scheme = 4
            elif self.model == 1 and self.diffusion_model != 0:
                self.time_scheme = 1
            elif self.model == 2:
                self.time_scheme = 5
            elif self.model == 3:
                self.time_scheme = 5

    @staticmethod
    def check_types(reference, data):
        errors = {}
        for key, value in data.items():
            if key not in reference:
                errors[key] = "unexpected key"
            elif not isinstance(value, type(reference[key])):
                errors[key] = (f"expected {type(reference[key]).__name__}, "
                               f"got {type(value).__name__}")
        if errors:
            raise TypeError(f"Failed initialization, type check failed with errors: {errors}")

    def check_values(self):
        bad = False
        if self.time_step < 0.:
            bad = True
        if self.model < 0 or self.model > 3:
            bad = True
        if self.model == 1:
            bad |= not (1 <= self.time_scheme <= 4)
        elif self.model == 2:
            if self.diffusion_model == 0:
                bad |= not (1 <= self.time_scheme <= 5)
            else:
                bad |= self.time_scheme not in (1, 5)
            bad |= not (1 <= self.diffusion_lsm2_option <= 3)
        elif self.model == 3:
            bad |= self.diffusion_model == 0
            bad |= self.time_scheme not in (1, 5)
        bad |= not (0 <= self.particle_velocity_init <= 1)
        bad |= not (1 <= self.rng_method <= 3)
        bad |= self.water_density < 0.
        bad |= not (0 <= self.diffusion_model <= 3)
        bad |= self.horizontal_diffusivity < 0. or self.vertical_diffusivity < 0.
        bad |= self.schmidt_number <= 0.
        bad |= not (1 <= self.diffusion_lsm2_option <= 3)
        bad |= self.diffusion_lsm3_tl_horizontal <= 0.
        bad |= self.diffusion_lsm3_tl_vertical <= 0.
        bad |= not (1 <= self.lsm3_edge_opt <= 2)
        bad |= self.max_wall_rebounds < 0
        bad |= not (1 <= self.boundary_conditions_type <= 2)
        bad |= not (0. <= self.rebound_damping_coef <= 1.)
        bad |= self.wall_roughness_angle < 0.
        bad |= not (0. <= self.stranding_probability <= 1.)
        bad |= self.listing_printout_period < 0 or self.output_printout_period < 0
        bad |= self.output_file_format not in ("txt", "vtk", "all")
        if bad:
            raise ValueError("Failed initialization, check parameters")
