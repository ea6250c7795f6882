"""Benchmark workloads of the batched, served, large and small configurations
(benchmarks/suite.py); bench.py imports the batched and served ones."""
