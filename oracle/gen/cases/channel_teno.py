"""Problem script: 3D compressible turbulent channel, TENO6 + metrics.

Written for this build against the reference's user API, following
apps/channel_flow/compressible_TCF_TENO/turbulent_channel.py: 3D Navier-Stokes with the power-law
viscosity mu = T^0.7 and the constant forcing c_j of the momentum (- c_i) and energy (- c_j u_j)
equations, periodic x0 and x2, isothermal walls on both x1 faces (default closures), metrics
stretched in x1 (tanh clustering at both walls), LLFTeno(6) with a fixed cut-off, StoreSome(4) central
derivatives, RungeKuttaLS(3, 'SSP'), the perturbed laminar-log profile initial condition.  The
statistics classes of the app are left out.  Grid size, dt and step count are run-time parameters.
"""
from sympy import sin, log, cos, pi, tanh
from opensbli import *
from opensbli.utilities.helperfunctions import substitute_simulation_parameters

ndim = 3
sc1 = "**{'scheme':'Teno'}"
mass = "Eq(Der(rho,t), - Conservative(rhou_j,x_j,%s))" % sc1
momentum = "Eq(Der(rhou_i,t) , -Conservative(rhou_i*u_j + KD(_i,_j)*p,x_j , %s) + Der(tau_i_j,x_j) - KD(_i,_j)*c_j )" % sc1
energy = "Eq(Der(rhoE,t), - Conservative((p+rhoE)*u_j,x_j, %s) - Der(q_j,x_j) + Der(u_i*tau_i_j ,x_j) - Dot(c_j, u_j))" % sc1
stress_tensor = "Eq(tau_i_j, (mu/Re)*(Der(u_i,x_j)+ Der(u_j,x_i) - (2/3)* KD(_i,_j)* Der(u_k,x_k)))"
heat_flux = "Eq(q_j, (-mu/((gama-1)*Minf*Minf*Pr*Re))*Der(T,x_j))"
substitutions = [stress_tensor, heat_flux]
constants = ["Re", "Pr", "gama", "Minf", "c_j"]
coordinate_symbol = "x"
velocity = "Eq(u_i, rhou_i/rho)"
pressure = "Eq(p, (gama-1)*(rhoE - rho*(1/2)*(KD(_i,_j)*u_i*u_j)))"
speed_of_sound = "Eq(a, (gama*p/rho)**0.5)"
temperature = "Eq(T, p*gama*Minf*Minf/(rho))"
viscosity = "Eq(mu, (T**0.7))"

ein = EinsteinEquation()
simulation_eq = SimulationEquations()
for e in (mass, momentum, energy):
    simulation_eq.add_equations(ein.expand(e, ndim, coordinate_symbol, substitutions, constants))
constituent = ConstituentRelations()
for e in (velocity, pressure, temperature, speed_of_sound, viscosity):
    constituent.add_equations(ein.expand(e, ndim, coordinate_symbol, substitutions, constants))

block = SimulationBlock(ndim, block_number=0)
local_dict = {"block": block, "GridVariable": GridVariable, "DataObject": DataObject}
dx, dy, dz = block.deltas
i, j, k = block.grid_indexes
gama, Minf, Re = symbols('gama Minf Re', **{'cls': ConstantObject})
q_vector = flatten(simulation_eq.time_advance_arrays)

for con in ["Minf", "Twall"]:
    local_dict[con] = ConstantObject(con)
rhoE_wall = parse_expr("Eq(DataObject(rhoE), DataObject(rho)*Twall/(gama*(gama-1.0)*Minf**2.0))", local_dict=local_dict)
boundaries = [PeriodicBC(0, side=0), PeriodicBC(0, side=1),
              IsothermalWallBC(1, 0, [rhoE_wall]), IsothermalWallBC(1, 1, [rhoE_wall]),
              PeriodicBC(2, 0), PeriodicBC(2, 1)]
block.set_block_boundaries(boundaries)

x, y, z = symbols('x0:%d' % ndim, **{'cls': DataObject})
ny = ConstantObject('block0np1')
stretch = ConstantObject('stretch')
Ly = 2
stretched = 0.5*Ly*(1.0-((tanh(stretch*(1.0-2.0*(j/(ny-1.0)))))/(tanh(stretch))))-1.0
grid_equations = [Eq(x, i * dx), Eq(y, stretched), Eq(z, k * dz)]
lx, ly, lz = symbols('lx0:%s' % ndim, **{'cls': ConstantObject})
sx, sy, sz = symbols('sx0:%s' % ndim, **{'cls': GridVariable})
cx, cy, cz = symbols('cx0:%s' % ndim, **{'cls': GridVariable})
ubar, amp, vonkar, b = symbols('ubar amp vonkar b', **{'cls': GridVariable})
ic = [Eq(b, 5.5), Eq(vonkar, 2.5)]
ic += [Eq(ubar, Piecewise(((1 - Abs(y)) * Re, (1 - Abs(y)) * Re < 10.0), (vonkar * log((1 - Abs(y)) * Re) + b, True)))]
ic += [Eq(amp, 0.1 * (vonkar * log(Re) + b))]
ic += [Eq(sx, sin(4.0 * pi * x / lx)), Eq(sy, sin(pi * y)), Eq(sz, sin(2.0 * pi * z / lz))]
ic += [Eq(cx, cos(4.0 * pi * x / lx)), Eq(cy, S.One + cos(pi * y)), Eq(cz, cos(2.0 * pi * z / lz))]
d, u, v, w, p = symbols('d u0 u1 u2 p', **{'cls': GridVariable})
ic += [Eq(u, ubar + amp * (lx / 2.0) * cx * sy * sz), Eq(v, - amp * sx * cy * sz),
       Eq(w, - amp * (lz / 2.0) * sx * sy * cz), Eq(p, S.One / (gama * Minf**2.0)), Eq(d, S.One)]
ic += [Eq(q_vector[0], d), Eq(q_vector[1], d * u), Eq(q_vector[2], d * v), Eq(q_vector[3], d * w),
       Eq(q_vector[4], p / (gama - S.One) + 0.5 * d * (u**2 + v**2 + w**2))]
initial = GridBasedInitialisation()
initial.add_equations(grid_equations + ic)

metriceq = MetricsEquation()
metriceq.generate_transformations(ndim, coordinate_symbol, [(False, False), (True, False), (False, False)], 2)
simulation_eq.apply_metrics(metriceq)
block.set_equations([constituent, simulation_eq, initial, metriceq])

schemes = {}
teno = LLFTeno(6, averaging=RoeAverage([0, 1]))
schemes[teno.name] = teno
cent = StoreSome(4, 'u0 u1 u2 T')
schemes[cent.name] = cent
rk = RungeKuttaLS(3, formulation='SSP')
schemes[rk.name] = rk
block.set_discretisation_schemes(schemes)

h5 = iohdf5(iotype="Write")
h5.add_arrays(simulation_eq.time_advance_arrays + [x, y, z, DataObject('D11')])
block.setio([h5])
block.discretise()
alg = TraditionalAlgorithmRK(block)
SimulationDataType.set_datatype(Double)
OPSC(alg)
constants = ['Re', 'gama', 'Minf', 'Pr', 'Twall', 'dt', 'niter', 'block0np0', 'block0np1', 'block0np2',
             'Delta0block0', 'Delta1block0', 'Delta2block0', "c0", "c1", "c2", "lx0", "lx2", "stretch", 'TENO_CT', 'eps']
values = ['190.71', '1.4', '0.0955', '0.7', '1.0', '0.0002', '250000', '64', '64', '32',
          '4.0*M_PI/block0np0', '2.0/(block0np1-1)', '(4.0*M_PI/3.0)/block0np2', '-1', '0', '0', "4.0*M_PI",
          "(4.0*M_PI/3.0)", "1.7", '1e-7', '1e-15']
substitute_simulation_parameters(constants, values)
