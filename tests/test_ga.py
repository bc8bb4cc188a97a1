"""The restated genetic algorithm (GA/ga_core.cpp) on CPU with a cheap fitness."""
import numpy as np

from randomwalk_nmr_gb300.ga import GeneticAlgorithm, correlation_fitness, misfit_fitness


def test_ga_converges_and_counts_evaluations():
    target = np.array([12.0, 30.0, 5.0])
    fit = lambda g: 1.0 / (1.0 + np.sum((g - target) ** 2))  # noqa: E731
    ga = GeneticAlgorithm(fit, [2, 2, 2], [40, 40, 40], population=64, seed=3)
    assert ga.evaluations == 64
    best, bf = ga.run(50)
    # 32 offspring per generation plus any diversity re-evaluations
    assert ga.evaluations >= 64 + 50 * 32
    assert np.all(np.abs(best - target) < 3.0) and bf > 0.05
    assert np.all(ga.fit[:-1] >= ga.fit[1:])  # sorted by fitness


def test_ga_is_reproducible_and_bounded():
    fit = lambda g: float(np.exp(-np.sum((g - 7.0) ** 2)))  # noqa: E731
    a = GeneticAlgorithm(fit, [1, 1], [10, 10], population=16, seed=9)
    b = GeneticAlgorithm(fit, [1, 1], [10, 10], population=16, seed=9)
    a.run(5)
    b.run(5)
    assert np.array_equal(a.genes, b.genes) and a.evaluations == b.evaluations
    assert np.all(a.genes >= 1) and np.all(a.genes <= 10)


def test_fitness_helpers():
    t = np.exp(-np.linspace(0, 3, 50))
    model = lambda g: np.exp(-g[0] * np.linspace(0, 3, 50))  # noqa: E731
    assert correlation_fitness(model, t)([1.0]) > 0.999999
    f = misfit_fitness(model, t, 1e-3)
    assert f([1.0]) == 1.0 and f([1.5]) < f([1.1])
