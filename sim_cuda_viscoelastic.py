"""Command-line twin of the reference backend script: ``python sim_cuda_viscoelastic.py -c cfg.json``.

Runs every (iteration, emission law) of the experiment on the GB300 stepper
(:class:`taichi_sim_gb300.backends.SimulatorCudaViscoelastic`); missing config keys and value
errors (Courant, stability) are reported as the reference's scripts do.
"""
import argparse

from taichi_sim_gb300.backends import SimulatorCudaViscoelastic


def main(argv=None):
    parser = argparse.ArgumentParser()
    parser.add_argument('-c', '--config', help='Configuration file', default='config.json')
    args = parser.parse_args(argv)
    sim = SimulatorCudaViscoelastic(args.config)
    try:
        sim.run()
    except KeyError as key:
        print(f"Chave {key} nao encontrada no arquivo de configuracao.")
    except ValueError as value:
        print(value)


if __name__ == "__main__":
    main()
