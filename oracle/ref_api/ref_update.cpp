// ref_update.cpp -- the reference's own explicit update() loops, driven from
// the command line (TEST INFRASTRUCTURE: builds golden vectors and pins the C
// oracle in pf_oracle.c; never part of the product).
//
// Compiled by oracle/Makefile against the reference's headers (MMSP.hpp:
// grid, laplacian, swap, ghostswap, input/output), without copying them.
// The bodies below keep the loop structure of
//   examples/phase_transitions/cahn-hilliard/explicit/cahn-hilliard.cpp:47-81
//   examples/coarsening/grain_growth/isotropic/phase_field/graingrowth.cpp:73-111
//   examples/phase_transitions/allen-cahn/allen-cahn.cpp:47-75
//   examples/coarsening/zener_pinning/isotropic/phase_field/zener.cpp:103-143
//   examples/coarsening/ostwald_ripening/isotropic/phase_field/ostwald.cpp:56-123
//   examples/phase_transitions/cahn-hilliard/convex_splitting/cahn-hilliard.cpp:273-463
//   examples/coarsening/grain_growth/isotropic/sparsePF/graingrowth.cpp:58-120
// The "shipped" models are those loops with the examples' own expressions;
// the "baseline" models substitute f(c)=c^2(1-c)^2 for Cahn-Hilliard and
// f = sum(-e^2/2+e^4/4) + gamma*sum_{i<j} e_i^2 e_j^2 for grain growth, with
// the parameters taken from the command line instead of being hard-coded.
//
// usage: ref_update MODEL IN.dat OUT.dat STEPS [params...]
//   ch_baseline      K M dt
//   ch_shipped       r u K M dt
//   ac_baseline      gamma kappa L dt
//   graingrowth      dt
//   zener            dt
//   ostwald          dt L D Calpha Cbeta A delta epsilon kappa
//   ch_convex        dt D K C0 Ca Cb A omega tolerance   (prints "iterations <n>" of the last step)
//   ac_scalar        r u K M dt
//   sparsepf         dt epsilon   (IN/OUT are sparse list files, see run_sparse)
// Prints "update_seconds <t>" (std::chrono around update() only).
#include "MMSP.hpp"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

namespace MMSP {

template <int dim> void ch_update(grid<dim, double>& oldGrid, int steps, bool shipped,
                                  const std::vector<double>& p)
{
	ghostswap(oldGrid);
	grid<dim, double> newGrid(oldGrid);
	grid<dim, double> temp(oldGrid);
	double r = 0, u = 0, K, M, dt;
	if (shipped) { r = p[0]; u = p[1]; K = p[2]; M = p[3]; dt = p[4]; }
	else { K = p[0]; M = p[1]; dt = p[2]; }
	for (int step = 0; step < steps; step++) {
		for (int i = 0; i < nodes(oldGrid); i++) {
			double phi = oldGrid(i);
			if (shipped)
				temp(i) = -r * phi + u * pow(phi, 3) - K * laplacian(oldGrid, i);
			else
				temp(i) = 2.0 * phi * (1.0 - phi) * (1.0 - 2.0 * phi) - K * laplacian(oldGrid, i);
		}
		ghostswap(temp);
		for (int i = 0; i < nodes(oldGrid); i++)
			newGrid(i) = oldGrid(i) + dt * M * laplacian(temp, i);
		swap(oldGrid, newGrid);
		ghostswap(oldGrid);
	}
}

template <int dim> void ac_scalar_update(grid<dim, double>& oldGrid, int steps,
                                         const std::vector<double>& p)
{
	ghostswap(oldGrid);
	grid<dim, double> newGrid(oldGrid);
	double r = p[0], u = p[1], K = p[2], M = p[3], dt = p[4];
	for (int step = 0; step < steps; step++) {
		for (int i = 0; i < nodes(oldGrid); i++) {
			double phi = oldGrid(i);
			newGrid(i) = phi - dt * M * (-r * phi + u * pow(phi, 3) - K * laplacian(oldGrid, i));
		}
		swap(oldGrid, newGrid);
		ghostswap(oldGrid);
	}
}

template <int dim> void gg_update(grid<dim, vector<double> >& oldGrid, int steps, bool shipped,
                                  const std::vector<double>& p)
{
	ghostswap(oldGrid);
	grid<dim, vector<double> > newGrid(oldGrid);
	double gamma = 0, kappa = 0, L = 0, dt;
	if (shipped) dt = p[0];
	else { gamma = p[0]; kappa = p[1]; L = p[2]; dt = p[3]; }
	for (int step = 0; step < steps; step++) {
		for (int i = 0; i < nodes(oldGrid); i++) {
			const vector<double>& phi = oldGrid(i);
			vector<double> lap = laplacian(oldGrid, i);
			double sum = 0.0;
			for (int j = 0; j < fields(oldGrid); j++)
				sum += phi[j] * phi[j];
			for (int j = 0; j < fields(oldGrid); j++) {
				if (shipped)
					newGrid(i)[j] = phi[j] - dt * (-phi[j] - pow(phi[j], 3) + 2.0 * (phi[j] * sum - lap[j]));
				else
					newGrid(i)[j] = phi[j] - dt * L * (-phi[j] + phi[j] * phi[j] * phi[j]
					                + 2.0 * gamma * phi[j] * (sum - phi[j] * phi[j])
					                - kappa * lap[j]);
			}
		}
		swap(oldGrid, newGrid);
		ghostswap(oldGrid);
	}
}

// examples/coarsening/zener_pinning/isotropic/phase_field/zener.cpp:103-143
// with dt from the command line.
template <int dim> void zener_update(grid<dim, vector<double> >& oldGrid, int steps,
                                     const std::vector<double>& p)
{
	ghostswap(oldGrid);
	grid<dim, vector<double> > newGrid(oldGrid);
	double dt = p[0];
	for (int step = 0; step < steps; step++) {
		for (int i = 0; i < nodes(oldGrid); i++) {
			vector<double> lap = laplacian(oldGrid, i);
			double sum = 0.0;
			for (int j = 0; j < fields(oldGrid); j++) {
				double phi = oldGrid(i)[j];
				sum += phi * phi;
			}
			for (int j = 0; j < fields(oldGrid); j++) {
				double phi = oldGrid(i)[j];
				if (j == 0) newGrid(i)[j] = phi;
				else newGrid(i)[j] = phi - dt * (-phi - pow(phi, 3) + 2.0 * (phi * sum - lap[j]));
			}
		}
		swap(oldGrid, newGrid);
		ghostswap(oldGrid);
	}
}

// examples/coarsening/ostwald_ripening/isotropic/phase_field/ostwald.cpp:56-123
// with dt, L, D, Calpha, Cbeta, A, delta, epsilon, kappa from the command line
// (the example's :66-80 constants by default).
template <int dim> void ostwald_update(grid<dim, vector<double> >& oldGrid, int steps,
                                       const std::vector<double>& p)
{
	ghostswap(oldGrid);
	grid<dim, vector<double> > newGrid(oldGrid);
	grid<dim, double> wspace(oldGrid, 1);
	double dt = p[0], L = p[1], D = p[2], Calpha = p[3], Cbeta = p[4], A = p[5], delta = p[6],
	       epsilon = p[7], kappa = p[8];
	double Cmatrix = 0.5 * (Calpha + Cbeta);
	double B = A / pow(Cbeta - Cmatrix, 2);
	double gamma = 2.0 / pow(Cbeta - Calpha, 2);
	double Dalpha = gamma / pow(delta, 2);
	double Dbeta = gamma / pow(delta, 2);
	for (int step = 0; step < steps; step++) {
		for (int n = 0; n < nodes(oldGrid); n++) {
			vector<int> x = position(oldGrid, n);
			double sum = 0.0;
			for (int i = 1; i < fields(oldGrid); i++)
				sum += pow(oldGrid(n)[i], 2);
			double C = oldGrid(n)[0];
			double lap = laplacian(oldGrid, x, 0);
			wspace(x) = -A * (C - Cmatrix) + B * pow(C - Cmatrix, 3)
			            + Dalpha * pow(C - Calpha, 3) + Dbeta * pow(C - Cbeta, 3)
			            - gamma * (C - Calpha) * sum - kappa * lap;
		}
		ghostswap(wspace);
		for (int n = 0; n < nodes(oldGrid); n++) {
			vector<int> x = position(oldGrid, n);
			double lap = laplacian(wspace, x);
			double C = oldGrid(n)[0];
			newGrid(n)[0] = C + dt * D * lap;
			double sum = 0.0;
			for (int i = 1; i < fields(oldGrid); i++)
				sum += pow(oldGrid(n)[i], 2);
			vector<double> vlap = laplacian(oldGrid, x);
			for (int i = 1; i < fields(oldGrid); i++) {
				double value = oldGrid(n)[i];
				newGrid(n)[i] = value - dt * L * (-gamma * pow(C - Calpha, 2) + delta * pow(value, 3)
				                                  + epsilon * value * (sum - pow(value, 2)) - kappa * vlap[i]);
			}
		}
		swap(oldGrid, newGrid);
		ghostswap(oldGrid);
	}
}

// examples/phase_transitions/cahn-hilliard/convex_splitting/cahn-hilliard.cpp:273-463
// (parametric free energy :38-96), constants from the command line; the two
// Laplacian helpers of that file (:135-170) restated.
template <int dim> double cs_field_laplacian(const grid<dim, vector<double> >& GRID, const vector<int>& x, int field)
{
	double laplacian = 0.0;
	vector<int> s = x;
	const double& y = GRID(x)[field];
	for (int i = 0; i < dim; i++) {
		s[i] += 1;
		const double& yh = GRID(s)[field];
		s[i] -= 2;
		const double& yl = GRID(s)[field];
		s[i] += 1;
		double weight = 1.0 / pow(dx(GRID, i), 2.0);
		laplacian += weight * (yh - 2.0 * y + yl);
	}
	return laplacian;
}

template <int dim> double cs_fringe_laplacian(const grid<dim, vector<double> >& GRID, const vector<int>& x, int field)
{
	double laplacian = 0.0;
	vector<int> s = x;
	for (int i = 0; i < dim; i++) {
		s[i] += 1;
		const double& yh = GRID(s)[field];
		s[i] -= 2;
		const double& yl = GRID(s)[field];
		s[i] += 1;
		double weight = 1.0 / pow(dx(GRID, i), 2.0);
		laplacian += weight * (yh + yl);
	}
	return laplacian;
}

template <int dim> void convex_update(grid<dim, vector<double> >& oldGrid, int steps, const std::vector<double>& p)
{
	double dt = p[0], D = p[1], K = p[2], C0 = p[3], Ca = p[4], Cb = p[5], A = p[6], omega = p[7],
	       tolerance = p[8];
	double B = A / pow(Ca - C0, 2.0);
	double QA = B + Ca + Cb;
	double QB = 3.0 * (B * C0 + Ca * Ca + Cb * Cb);
	double QC = 3.0 * (B * C0 * C0 + pow(Ca, 3.0) + pow(Cb, 3.0));
	double QD = B * pow(C0, 3.0) + pow(Ca, 4.0) + pow(Cb, 4.0);
	unsigned int residual_step = 5, max_iter = 10000;
	ghostswap(oldGrid);
	grid<dim, vector<double> > newGrid(oldGrid);
	newGrid.copy(oldGrid);
	double gridSize = static_cast<double>(nodes(oldGrid));
	double lapWeight = 0.0;
	for (int d = 0; d < dim; d++)
		lapWeight += 2.0 / pow(dx(oldGrid, d), 2.0);
	unsigned int iter = 0;
	for (int step = 0; step < steps; step++) {
		double residual = 1.0;
		iter = 0;
		ghostswap(oldGrid);
		ghostswap(newGrid);
		while (iter < max_iter && residual > tolerance) {
			for (int color = 1; color > -1; color--) {
				for (int n = 0; n < nodes(oldGrid); n++) {
					vector<int> x = position(oldGrid, n);
					int x_sum = 0;
					for (int d = 0; d < dim; d++)
						x_sum += x[d];
					if (x_sum % 2 == color)
						continue;
					double cOld = oldGrid(n)[0];
					double cGuess = newGrid(n)[0];
					double uGuess = newGrid(n)[1];
					double A12 = dt * D * lapWeight;
					double A21 = -(QA * pow(newGrid(n)[0], 2.0) + QC) - K * lapWeight;
					double detA = 1.0 - (A12 * A21);
					double B1 = cOld + D * dt * cs_fringe_laplacian(newGrid, x, 1);
					double B2 = (-A * (cOld - C0) - QB * pow(cOld, 2.0) - QD) - K * cs_fringe_laplacian(newGrid, x, 0);
					double cNew = (B1 - B2 * A12) / detA;
					double uNew = (B2 - B1 * A21) / detA;
					newGrid(n)[0] = omega * cNew + (1.0 - omega) * cGuess;
					newGrid(n)[1] = omega * uNew + (1.0 - omega) * uGuess;
				}
				ghostswap(newGrid);
			}
			iter++;
			if (iter < residual_step || iter % residual_step == 0) {
				double normB = 0.0;
				residual = 0.0;
				for (int n = 0; n < nodes(oldGrid); n++) {
					vector<int> x = position(oldGrid, n);
					double lapC = cs_field_laplacian(newGrid, x, 0);
					double lapU = cs_field_laplacian(newGrid, x, 1);
					double cOld = oldGrid(n)[0];
					double cNew = newGrid(n)[0];
					double uNew = newGrid(n)[1];
					double B1 = cOld;
					double B2 = -A * (cOld - C0) - QB * pow(cOld, 2.0) - QD;
					double AX1 = cNew - D * dt * lapU;
					double AX2 = uNew - (QA * pow(cNew, 3.0) + QC * cNew) + K * lapC;
					double R1 = B1 - AX1;
					double R2 = B2 - AX2;
					double error = R1 * R1 + R2 * R2;
					residual += error;
					normB += B1 * B1 + B2 * B2;
				}
				residual = sqrt(residual / normB) / (2.0 * gridSize);
			}
		}
		if (iter == max_iter) {
			std::cerr << "solver stagnated on step " << step << std::endl;
			std::exit(3);
		}
		swap(oldGrid, newGrid);
	}
	std::printf("iterations %u\n", iter);
}

// examples/coarsening/grain_growth/isotropic/sparsePF/graingrowth.cpp:58-120 with dt and
// epsilon from the command line, on the reference's grid<dim,sparse<double> >.
template <int dim> void sparse_update(grid<dim, sparse<double> >& oldGrid, int steps,
                                      const std::vector<double>& p)
{
	ghostswap(oldGrid);
	grid<dim, sparse<double> > newGrid(oldGrid);
	const double dt = p[0];
	const double epsilon = p[1];
	for (int step = 0; step < steps; step++) {
		for (int n = 0; n < nodes(oldGrid); n++) {
			vector<int> x = position(oldGrid, n);
			sparse<bool> neighbors;
			for (int j = 0; j < dim; j++)
				for (int k = -1; k <= 1; k++) {
					x[j] += k;
					for (int h = 0; h < length(oldGrid(x)); h++) {
						int i = index(oldGrid(x), h);
						set(neighbors, i) = 1;
					}
					x[j] -= k;
				}
			if (length(neighbors) < 2)
				newGrid(n) = oldGrid(n);
			else {
				sparse<double> lap = laplacian(oldGrid, n);
				double sum = 0.0;
				for (int j = 0; j < length(oldGrid(n)); j++) {
					double phi = value(oldGrid(n), j);
					sum += phi * phi;
				}
				for (int j = 0; j < length(neighbors); j++) {
					int i = index(neighbors, j);
					double phi = oldGrid(n)[i];
					double v = phi - dt * (-phi - pow(phi, 3) + 2.0 * (phi * sum - lap[i]));
					if (v > epsilon) set(newGrid(n), i) = v;
				}
			}
		}
		swap(oldGrid, newGrid);
		ghostswap(oldGrid);
	}
}

} // namespace MMSP

// Sparse grids travel as a plain binary list file (not the MMSP grid format, whose item
// padding bytes are uninitialised): int32 dim, int32 n[dim], then per cell in node order
// int32 count and count x (int32 index, float64 value).
template <int dim> MMSP::grid<dim, MMSP::sparse<double> >* make_sparse_grid(const int* n);
template <> MMSP::grid<1, MMSP::sparse<double> >* make_sparse_grid<1>(const int* n)
{
	return new MMSP::grid<1, MMSP::sparse<double> >(0, 0, n[0]);
}
template <> MMSP::grid<2, MMSP::sparse<double> >* make_sparse_grid<2>(const int* n)
{
	return new MMSP::grid<2, MMSP::sparse<double> >(0, 0, n[0], 0, n[1]);
}
template <> MMSP::grid<3, MMSP::sparse<double> >* make_sparse_grid<3>(const int* n)
{
	return new MMSP::grid<3, MMSP::sparse<double> >(0, 0, n[0], 0, n[1], 0, n[2]);
}

static double now_s();

template <int dim> int run_sparse(std::ifstream& in, const char* out, int steps, const std::vector<double>& p)
{
	int n[3] = {1, 1, 1};
	in.read(reinterpret_cast<char*>(n), sizeof(int) * dim);
	MMSP::grid<dim, MMSP::sparse<double> >* g = make_sparse_grid<dim>(n);
	for (int i = 0; i < MMSP::nodes(*g); i++) {
		int count = 0;
		in.read(reinterpret_cast<char*>(&count), sizeof(int));
		for (int h = 0; h < count; h++) {
			int index = 0;
			double v = 0.0;
			in.read(reinterpret_cast<char*>(&index), sizeof(int));
			in.read(reinterpret_cast<char*>(&v), sizeof(double));
			MMSP::set((*g)(i), index) = v;
		}
	}
	if (!in) {
		delete g;
		return 4;
	}
	double t0 = now_s();
	MMSP::sparse_update(*g, steps, p);
	double t1 = now_s();
	std::printf("update_seconds %.9f\n", t1 - t0);
	std::ofstream o(out, std::ios::binary);
	int d = dim;
	o.write(reinterpret_cast<const char*>(&d), sizeof(int));
	o.write(reinterpret_cast<const char*>(n), sizeof(int) * dim);
	for (int i = 0; i < MMSP::nodes(*g); i++) {
		const MMSP::sparse<double>& s = (*g)(i);
		int count = MMSP::length(s);
		o.write(reinterpret_cast<const char*>(&count), sizeof(int));
		for (int h = 0; h < count; h++) {
			int index = MMSP::index(s, h);
			double v = MMSP::value(s, h);
			o.write(reinterpret_cast<const char*>(&index), sizeof(int));
			o.write(reinterpret_cast<const char*>(&v), sizeof(double));
		}
	}
	delete g;
	return o ? 0 : 4;
}

static double now_s()
{
	using namespace std::chrono;
	return duration<double>(steady_clock::now().time_since_epoch()).count();
}

template <int dim> int run_scalar(const std::string& model, const char* in, const char* out,
                                  int steps, const std::vector<double>& p)
{
	MMSP::grid<dim, double> g(in);
	double t0 = now_s();
	if (model == "ch_baseline") MMSP::ch_update(g, steps, false, p);
	else if (model == "ch_shipped") MMSP::ch_update(g, steps, true, p);
	else if (model == "ac_scalar") MMSP::ac_scalar_update(g, steps, p);
	else return 2;
	double t1 = now_s();
	std::printf("update_seconds %.9f\n", t1 - t0);
	MMSP::output(g, out);
	return 0;
}

template <int dim> int run_vector(const std::string& model, const char* in, const char* out,
                                  int steps, const std::vector<double>& p)
{
	MMSP::grid<dim, MMSP::vector<double> > g(in);
	double t0 = now_s();
	if (model == "ac_baseline") MMSP::gg_update(g, steps, false, p);
	else if (model == "graingrowth") MMSP::gg_update(g, steps, true, p);
	else if (model == "zener") MMSP::zener_update(g, steps, p);
	else if (model == "ostwald") MMSP::ostwald_update(g, steps, p);
	else if (model == "ch_convex") MMSP::convex_update(g, steps, p);
	else return 2;
	double t1 = now_s();
	std::printf("update_seconds %.9f\n", t1 - t0);
	MMSP::output(g, out);
	return 0;
}

int main(int argc, char* argv[])
{
	if (argc < 5) {
		std::cerr << "usage: ref_update MODEL IN OUT STEPS [params...]" << std::endl;
		return 1;
	}
	std::string model = argv[1];
	int steps = std::atoi(argv[4]);
	std::vector<double> p;
	for (int i = 5; i < argc; i++) p.push_back(std::atof(argv[i]));
	size_t need = (model == "ch_baseline") ? 3 : (model == "ch_shipped" || model == "ac_scalar") ? 5
	            : (model == "ac_baseline") ? 4 : (model == "graingrowth" || model == "zener") ? 1
	            : (model == "ostwald" || model == "ch_convex") ? 9 : (model == "sparsepf") ? 2 : 0;
	if (need == 0 || p.size() != need) {
		std::cerr << "bad model or parameter count" << std::endl;
		return 1;
	}
	if (model == "sparsepf") {
		std::ifstream in(argv[2], std::ios::binary);
		int d = 0;
		in.read(reinterpret_cast<char*>(&d), sizeof(int));
		int rc = d == 1 ? run_sparse<1>(in, argv[3], steps, p) : d == 2 ? run_sparse<2>(in, argv[3], steps, p)
		       : d == 3 ? run_sparse<3>(in, argv[3], steps, p) : 2;
		if (rc) std::cerr << "sparse list file could not be read or written" << std::endl;
		return rc;
	}
	std::ifstream hdr(argv[2]);
	std::string type;
	int dim = 0;
	std::getline(hdr, type);
	hdr >> dim;
	hdr.close();
	bool vec = type.find("vector") != std::string::npos;
	int rc = 2;
	if (vec) {
		if (dim == 1) rc = run_vector<1>(model, argv[2], argv[3], steps, p);
		if (dim == 2) rc = run_vector<2>(model, argv[2], argv[3], steps, p);
		if (dim == 3) rc = run_vector<3>(model, argv[2], argv[3], steps, p);
	} else {
		if (dim == 1) rc = run_scalar<1>(model, argv[2], argv[3], steps, p);
		if (dim == 2) rc = run_scalar<2>(model, argv[2], argv[3], steps, p);
		if (dim == 3) rc = run_scalar<3>(model, argv[2], argv[3], steps, p);
	}
	if (rc) std::cerr << "model/type mismatch: " << model << " on " << type << std::endl;
	return rc;
}
