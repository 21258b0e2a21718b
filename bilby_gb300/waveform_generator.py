"""A ``WaveformGenerator`` with bilby's interface
(bilby/gw/waveform_generator.py:12-300) for use without bilby installed.
bilby's own ``WaveformGenerator`` is accepted by the likelihood as well."""
from __future__ import annotations

import inspect

import numpy as np

from .conversion import convert_to_lal_binary_black_hole_parameters


def _model_args(model):
    params = list(inspect.signature(model).parameters.values())[1:]
    return {p.name for p in params if p.kind not in (p.VAR_KEYWORD, p.VAR_POSITIONAL)}


class WaveformGenerator:
    def __init__(self, duration=None, sampling_frequency=None, start_time=0, frequency_domain_source_model=None,
                 time_domain_source_model=None, parameters=None, parameter_conversion=None,
                 waveform_arguments=None):
        if time_domain_source_model is not None and frequency_domain_source_model is None:
            raise NotImplementedError("only frequency-domain source models are supported")
        self.duration = duration
        self.sampling_frequency = sampling_frequency
        self.start_time = start_time
        self.frequency_domain_source_model = frequency_domain_source_model
        self.time_domain_source_model = time_domain_source_model
        self.parameter_conversion = (convert_to_lal_binary_black_hole_parameters if parameter_conversion is None
                                     else parameter_conversion)
        self.waveform_arguments = dict(waveform_arguments or {})
        self.source_parameter_keys = _model_args(frequency_domain_source_model)
        self._cache = dict(parameters=None, waveform=None)
        self.use_cache = True

    @property
    def frequency_array(self):
        n_samples = np.round(self.duration * self.sampling_frequency)
        return np.linspace(0, self.sampling_frequency / 2, num=int(np.round(n_samples / 2) + 1))

    def _format_parameters(self, parameters):
        """waveform_generator.py:260-269."""
        new = dict(parameters)
        new, _ = self.parameter_conversion(new)
        for key in self.source_parameter_keys.symmetric_difference(new):
            new.pop(key)
        new.update(self.waveform_arguments)
        return new

    def frequency_domain_strain(self, parameters=None):
        if parameters is None:
            parameters = self._cache["parameters"]
        if self.use_cache and self._cache["parameters"] is not None and parameters == self._cache["parameters"]:
            return self._cache["waveform"]
        self._cache["parameters"] = dict(parameters)
        out = self.frequency_domain_source_model(self.frequency_array, **self._format_parameters(parameters))
        self._cache["waveform"] = out
        return out

    @property
    def meta_data(self):
        return dict(domain="frequency", frequency_domain_source_model=self.frequency_domain_source_model,
                    parameter_conversion=self.parameter_conversion, waveform_arguments=self.waveform_arguments)

    def __repr__(self):
        name = getattr(self.frequency_domain_source_model, "__name__", None)
        return (f"WaveformGenerator(duration={self.duration}, sampling_frequency={self.sampling_frequency}, "
                f"start_time={self.start_time}, frequency_domain_source_model={name}, "
                f"waveform_arguments={self.waveform_arguments})")
