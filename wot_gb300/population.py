"""Population — a measure over the cells of one day (wot/population.py:6-67)."""
from __future__ import annotations

import numpy as np


class Population:
    """A measure ``p`` over the cells at ``time`` (not necessarily summing to 1)."""

    def __init__(self, time, p, name=None):
        self.time = time
        self.p = np.asarray(p, dtype=np.float64)
        self.name = name

    def normalize(self):
        """Make the measure a probability distribution (:25-29)."""
        self.p = self.p / self.p.sum()

    def make_binary(self):
        """Set non-zero values to 1 (:31-37)."""
        p = np.zeros(len(self.p))
        p[self.p > 0.0] = 1.0
        self.p = p

    @staticmethod
    def get_missing_population(*populations):
        """The 'Other' population of cells no population covers (:39-47)."""
        initial_p_sum = np.array([pop.p for pop in populations]).T.sum(axis=1)
        missing_cells = np.where(initial_p_sum == 0)[0]
        if len(missing_cells) > 0:
            missing_cells_p = np.zeros_like(populations[0].p)
            missing_cells_p[missing_cells] = 1.0
            return Population(populations[0].time, missing_cells_p, 'Other')
        return None

    @staticmethod
    def copy(*populations, normalize=None, add_missing=False):
        """Copies, optionally plus 'Other', then normalised (True) or binary (False) (:49-67)."""
        populations = [Population(pop.time, pop.p, pop.name) for pop in populations]
        if add_missing:
            missing_pop = Population.get_missing_population(*populations)
            if missing_pop is not None:
                populations.append(missing_pop)
        if normalize or normalize == False:  # noqa: E712  (the reference's test: None means neither)
            for pop in populations:
                if normalize:
                    pop.normalize()
                else:
                    pop.make_binary()
        return populations
