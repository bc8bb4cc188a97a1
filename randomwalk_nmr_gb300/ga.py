"""The reference's genetic-algorithm relaxivity fit, restated (GA/ga_core.cpp, GA/individual.cpp,
GA/ga_defs.h), as the baseline the gradient fits are compared with.

The reference GA is not part of its build (src/backend/CMakeLists.txt comments it out) and calls
simulation methods that no longer exist (GA/ga_core.cpp:463-506), so it cannot be run; this is a
restatement of its algorithm:
  * population of real-valued genotypes initialised uniformly within bounds (createNewPopulation);
  * roulette-wheel parent selection on fitness, second parent different from the first
    (createParentsList, rouletteWheelSelection);
  * blend crossover with alpha ~ U(0, gamma) per gene (applyCrossover, "paper recommendation");
  * mutation: each gene with probability mutation_ratio moves by gene * deviation * U(-1, 1)
    (Individual::mutate), then clamped to the bounds (applyBounds);
  * offspring replace the worst individuals; the population is sorted by fitness
    (createNextGeneration, sortPopulation);
  * diversity control: if the mean normalised gene deviation drops below 1 - diversity, mutate
    every gene of the second to middle individuals, and after mutations_per_reset such
    impositions keep the top 25 % and re-draw the rest (checkGenotypeDeviation,
    applyGeneDiversification, imposeMutation, resetPopulation).
The reference draws every random number from a freshly seeded std::random_device; this restatement
uses one seeded generator so runs are reproducible. Its fitness (squared correlation of Laplace-
inverted T2 distributions) needs the Eigen-based inverter the reference keeps outside this path;
here the fitness is the squared correlation of the echo trains themselves.
"""
from __future__ import annotations

import numpy as np


class GeneticAlgorithm:
    def __init__(self, fitness, lo, hi, population=64, offspring_proportion=0.5, gamma=0.5, mutation_ratio=0.1,
                 mutation_deviation=1.0, mutations_per_reset=5, top_size=0.25, diversity=0.9, seed=0):
        self.fitness_fn = fitness
        self.lo = np.asarray(lo, np.float64)
        self.hi = np.asarray(hi, np.float64)
        self.P = int(population)
        self.n_off = int(round(self.P * offspring_proportion))
        self.n_off -= self.n_off % 2
        self.gamma = gamma
        self.mratio = mutation_ratio
        self.mdev = mutation_deviation
        self.m_per_reset = mutations_per_reset
        self.top = top_size
        self.diversity = diversity
        self.rng = np.random.default_rng(seed)
        self.evaluations = 0
        self.mutations_imposed = 0
        G = len(self.lo)
        self.genes = self.lo + (self.hi - self.lo) * self.rng.random((self.P, G))
        self.fit = np.array([self._eval(g) for g in self.genes])
        self._sort()
        self.best = (self.genes[0].copy(), self.fit[0])

    def _eval(self, g):
        self.evaluations += 1
        return float(self.fitness_fn(g))

    def _sort(self):
        order = np.argsort(-self.fit, kind="stable")
        self.genes, self.fit = self.genes[order], self.fit[order]
        if self.fit[0] > getattr(self, "best", (None, -np.inf))[1]:
            self.best = (self.genes[0].copy(), self.fit[0])

    def _roulette(self, p):
        c = np.cumsum(p)
        r = self.rng.random()
        idx = 0
        while idx < len(c) - 1 and r > c[idx]:
            idx += 1
        return idx

    def _mutate(self, g, ratio):
        flag = self.rng.random(len(g)) < ratio
        g = g + np.where(flag, g * self.mdev * self.rng.uniform(-1.0, 1.0, len(g)), 0.0)
        return g

    def generation(self):
        s = self.fit.sum()
        p = self.fit / s if s != 0 else self.fit
        children = []
        for _ in range(self.n_off // 2):
            a = self._roulette(p)
            b = self._roulette(p)
            tries = 0
            while b == a and tries < 1000:
                b = self._roulette(p)
                tries += 1
            alpha = self.rng.uniform(0.0, self.gamma, self.genes.shape[1])
            c1 = alpha * self.genes[a] + (1 - alpha) * self.genes[b]
            c2 = alpha * self.genes[b] + (1 - alpha) * self.genes[a]
            children += [c1, c2]
        children = [np.clip(self._mutate(c, self.mratio), self.lo, self.hi) for c in children]
        cfit = np.array([self._eval(c) for c in children])
        keep = self.P - len(children)
        self.genes = np.concatenate([self.genes[:keep], np.array(children)])
        self.fit = np.concatenate([self.fit[:keep], cfit])
        self._sort()
        # diversity control
        dev = np.mean(np.std(self.genes, axis=0) / np.mean(self.genes, axis=0))
        if dev < 1.0 - self.diversity:
            if self.mutations_imposed == self.m_per_reset:
                top = int(np.ceil(self.top * self.P))
                new = self.lo + (self.hi - self.lo) * self.rng.random((self.P - top, len(self.lo)))
                self.genes = np.concatenate([self.genes[:top], new])
                self.fit = np.concatenate([self.fit[:top], [self._eval(g) for g in new]])
                self.mutations_imposed = 0
            else:
                for i in range(1, self.P // 2):
                    self.genes[i] = np.clip(self._mutate(self.genes[i], 1.0), self.lo, self.hi)
                    self.fit[i] = self._eval(self.genes[i])
                self.mutations_imposed += 1
            self._sort()

    def run(self, generations):
        for _ in range(generations):
            self.generation()
        return self.best


def correlation_fitness(model, target):
    """Squared Pearson correlation of a model echo train with the target (the reference's fitness is
    the squared correlation of T2 distributions; GA/ga_core.cpp:463-476)."""
    target = np.asarray(target, np.float64)

    def f(genes):
        m = np.asarray(model(genes), np.float64)
        c = np.corrcoef(m, target)[0, 1]
        return 0.0 if not np.isfinite(c) else c * c

    return f


def misfit_fitness(model, target, sigma):
    """Positive fitness 1 / (1 + mean squared misfit / sigma^2) of a model echo train."""
    target = np.asarray(target, np.float64)

    def f(genes):
        m = np.asarray(model(genes), np.float64)
        return 1.0 / (1.0 + np.mean((m - target) ** 2) / (sigma * sigma))

    return f
