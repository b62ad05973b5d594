"""2D host model and experiment driver (``Simulator``).

Mirrors sim_support/simulator.py of the reference: ``Simulator(file_config,
sim_model, sim_type)`` builds every table (see :mod:`._model`), ``run()``
repeats ``implementation()`` for ``n_iter`` iterations times every emission
law and reports/saves the results (reference :321-605), and backends
subclass it and override ``implementation()`` (reference :608-611), which
returns a dict with the final field, the receiver traces, a device string
and the step-loop time.

``run()`` here is headless: the reference's matplotlib figures and Qt live
view need a graphics stack, so figures are produced only when matplotlib is
importable, and the live view (sim_taichi_elastic.py:320-329,
sim_support/windows_qt.py) is replaced by field snapshots: with
``show_anim`` (or ``save_snapshots``) set, a backend returns the ROI of the
field at every step the live view would show (``it % it_display == 0`` or
``it == 5``, 1-based) under ``"snapshots"``/``"snapshot_steps"``, and
``run()`` saves them next to the other results.  Result files keep the
reference's names.
"""
import os.path
from datetime import datetime
from time import time

import numpy as np

from ._model import ModelBase


def snapshot_steps(n_steps, it_display):
    """The 1-based steps after which the reference's live view shows the
    field: ``it % it_display == 0`` or ``it == 5``
    (sim_taichi_elastic.py:320, sim_webgpu_viscoelastic.py:519)."""
    every = max(1, int(it_display))
    steps = set(range(every, int(n_steps) + 1, every))
    if n_steps >= 5:
        steps.add(5)
    return sorted(steps)


def _field_and_traces(results):
    """The result dict's field and traces under either key convention.

    Elastic (Taichi-like) backends return ``pressure``/``sens_pressure``,
    viscoelastic ones ``stress``/``sens_stress``.
    """
    if "stress" in results:
        return results["stress"], results["sens_stress"]
    return results["pressure"], results["sens_pressure"]


class ExperimentDriver:
    """``run()``/``implementation()`` shared by the 2D and 3D models."""

    def _roi_crop(self, field):
        roi = self._roi
        if field.ndim == 2:
            return field[roi.get_ix_min():roi.get_ix_max(), roi.get_iz_min():roi.get_iz_max()]
        return field[roi.get_ix_min():roi.get_ix_max(), :, roi.get_iz_min():roi.get_iz_max()]

    def run(self, batched=False):
        """Run every (iteration, emission law) and report; returns the last result dict.

        ``batched=True`` (an extension) computes the emission laws of an
        iteration together, as shots of one batched launch
        (``implementation_batched``), each law with its own delays; the
        per-law loop, like the reference's, calls ``set_t0`` but injects the
        source term the constructor built."""
        now = datetime.now()
        sim_times, total_times, mse_values = list(), list(), list()
        results = dict()
        reflected_energy = reflected_energy_field = float("nan")
        result_dir = getattr(self, "_results_dir", os.path.join("."))
        for n in range(self._n_iter):
            print(f'Iteracao {n}')
            n_laws = self._emission_laws.shape[0] if hasattr(self, "_emission_laws") else 1
            if batched:
                t_start = time()
                batch_results = self.implementation_batched(
                    list(self._emission_laws) if hasattr(self, "_emission_laws") else [None])
                t_batch = time() - t_start
            for law in range(n_laws):
                print(f'\tLaw {law} of {n_laws}')
                if batched:
                    results = batch_results[law]
                    total_times.append(t_batch / n_laws)
                else:
                    if hasattr(self, "_emission_laws"):
                        for p in self._probes:
                            p.set_t0(self._emission_laws[law])
                    t_start = time()
                    results = self.implementation()
                    total_times.append(time() - t_start)
                sim_times.append(results["sim_time"])
                print(results["gpu_str"])
                print(f'{sim_times[-1]:.3}s')
                print(f'Tempo total (inclui transferencia de dados): {total_times[-1]:.3}s')
                name = os.path.join(result_dir, f'result_{self._name}_{now.strftime("%Y%m%d-%H%M%S")}_'
                                                f'{self._nx}x{self._ny}_{self._n_steps}_iter_{n}_law_{law}')
                field, traces = _field_and_traces(results)
                if self._dims == 2:
                    row = traces[self._n_steps - self.cpml_time, :] if 0 < self.cpml_time <= self._n_steps else traces[-1]
                    reflected_energy = (row ** 2).sum() * self._dt
                    print(f"Energia refletida (sensor): {reflected_energy:.2}")
                    reflected_energy_field = (field ** 2).sum() * self._dx * self._dy
                    print(f"Energia ultimo frame: {reflected_energy_field:.2}")
                mse = self._compare_with_reference(result_dir, field, traces)
                if mse is not None:
                    mse_values.append(mse)
                kind = "pressure" if self._sim_type == "acoustic" else "stress"
                if self._save_results and self._save_field:
                    np.save(name + ('_field_pressure' if kind == "pressure" else '_field_stress_yy'), field)
                if self._save_bscan:
                    np.save(name + f'_bscan_{kind}', traces)
                if "snapshots" in results:   # the live view's frames, headless
                    np.save(name + f'_snapshots_{kind}', results["snapshots"])
                    np.save(name + '_snapshot_steps', np.asarray(results["snapshot_steps"], np.int32))
                self._maybe_plot(law, field, traces, name, kind)

        sim_times, total_times = np.array(sim_times), np.array(total_times)
        mse_values = np.array(mse_values)
        print(f'TEMPO - {self._n_steps} pontos de tempo')
        if self._n_iter > 5:
            print(f'Tempo medio de execucao: {sim_times[5:].mean():.3}s (std = {sim_times[5:].std():.4})')
            print(f'Tempo medio total (inclui transferencia de dados): {total_times[5:].mean():.3}s '
                  f'(std = {total_times[5:].std():.4})')
        if self._save_sources:
            np.save(os.path.join(result_dir, f'sources_{self._name}_{now.strftime("%Y%m%d-%H%M%S")}'),
                    self._source_term)
        if self._save_results:
            base = os.path.join(result_dir, f'result_{self._name}_{now.strftime("%Y%m%d-%H%M%S")}_'
                                            f'{self._nx}x{self._ny}_{self._n_steps}_iter_{self._n_iter - 1}_')
            np.savetxt(base + 'GPU_.csv', sim_times, '%10.3f', delimiter=',')
            with open(base + '_desc.txt', 'w') as f:
                f.write('Parametros do ensaio\n--------------------\n\n')
                f.write(f'Simulador: {self._name}\n')
                f.write(f'Modelo do simulador: {self._sim_model}\n')
                f.write(f'Quantidade de iteracoes no tempo: {self._n_steps}\n')
                f.write(f'Tamanho da ROI: {self._nx}x{self._ny}\n')
                f.write(f'GPU: {results.get("gpu_str", "")}\n')
                f.write(f'Numero de simulacoes: {self._n_iter}\n')
                f.write(f"Energia refletida (sensor): {reflected_energy:.2}\n")
                f.write(f"Energia ultimo frame: {reflected_energy_field:.2}\n")
                if "msg_impl" in results:
                    f.write(results["msg_impl"])
                if self._n_iter > 5:
                    f.write(f'Tempo medio de execucao: {sim_times[5:].mean():.3}s\n')
                    f.write(f'Desvio padrao: {sim_times[5:].std():.4}\n')
                    f.write(f'Tempo medio total (inclui transferencia de dados): {total_times[5:].mean():.3}s\n')
                    f.write(f'Desvio padrao: {total_times[5:].std():.4}\n')
                else:
                    f.write(f'Tempo execucao: {sim_times[-1]:.3}s\n')
                    f.write(f'Tempo total (inclui transferencia de dados): {total_times[-1]:.3}s\n')
                    if mse_values.shape[0] > 0:
                        f.write(f'MSE do campo de pressao: {mse_values[-1, 0]:.4}\n')
                        f.write(f'MSE medio dos sensores de pressao: {mse_values[-1, 1]:.4}\n')
        return results

    def _compare_with_reference(self, result_dir, field, traces):
        """MSE against stored ``result_ref_<model>_{field,bscan}_pressure.npy`` if present."""
        try:
            ref_field = np.load(os.path.join(result_dir, f"result_ref_{self._sim_model}_field_pressure.npy"))
            ref_traces = np.load(os.path.join(result_dir, f"result_ref_{self._sim_model}_bscan_pressure.npy"))
        except FileNotFoundError as err:
            print(f"Arquivo {err} nao encontrado. Nao pode ser feita a comparacao com a referencia.")
            return None
        a, b = self._roi_crop(ref_field), self._roi_crop(field)
        mse_f = float(np.mean((a - b) ** 2)) if a.shape == b.shape else np.inf
        mse_t = float(np.mean((ref_traces - traces) ** 2)) if ref_traces.shape == traces.shape else np.inf
        print(f"MSE do campo de pressao em relacao a referencia: {mse_f:.4}")
        print(f"MSE dos sensores de pressao em relacao a referencia: {mse_t:.4}")
        return [mse_f, mse_t]

    def _maybe_plot(self, law, field, traces, name, kind):
        if not (self._plot_results or self._plot_bscan):
            return
        try:
            import matplotlib
            matplotlib.use("Agg")
            import matplotlib.pyplot as plt
        except ImportError:
            print("matplotlib nao disponivel: figuras omitidas")
            return
        if self._plot_bscan:
            fig = plt.figure()
            plt.title(f'{self._name} simulation B-scan {kind} - law({law})\n({self._nx}x{self._ny})')
            plt.imshow(traces, aspect='auto', cmap='viridis')
            plt.colorbar()
            if self._save_bscan:
                fig.savefig(name + f'_bscan_{kind}.png')
            plt.close(fig)
        if self._plot_results:
            img = self._roi_crop(field)
            img = img if img.ndim == 2 else img[:, img.shape[1] // 2, :]
            fig = plt.figure()
            plt.title(f'{self._name} simulation {kind} - law ({law})\n({self._nx}x{self._ny})')
            plt.imshow(img.T, aspect='auto', cmap='gray')
            plt.colorbar()
            if self._save_results:
                fig.savefig(name + f'_field_{kind}.png')
            plt.close(fig)

    def implementation(self):
        """Backends override this; the base only announces the run."""
        print(f'Simulacao {self._name}')
        return dict()

    def implementation_batched(self, laws):
        """One result dict per emission law (``None``: the probes' current
        delays), all laws computed together; backends that batch override it."""
        raise NotImplementedError(f"{type(self).__name__} has no batched run")


class Simulator(ExperimentDriver, ModelBase):
    """2D model: grid ``(nx, ny)`` with y the ROI height axis."""

    _dims = 2


__all__ = ["Simulator", "ExperimentDriver", "snapshot_steps"]
