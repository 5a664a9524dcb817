"""Problem script: 3D transitional shock-wave/boundary-layer interaction with a spanwise-periodic
body-force perturbation.

Written for this build against the reference's user API, following
apps/transitional_SBLI/transitional_SBLI.py: 3D Navier-Stokes with Sutherland viscosity, metrics
stretched in x1, TENO6 with the cut-off adapted by the metric-transformed Ducros sensor (stored as
TENO), StoreSome(4, 'u0 u1 u2') central derivatives, RungeKuttaLS(3), the body force
BF = A exp(-((x0-xF)^2 + (x1-yF)^2)) cos(bta x2) sin(omega dt iter) added to the continuity
equation, pressure-extrapolation inlet, extrapolation outlet, isothermal wall, shock-generator
Dirichlet top face (rhoE carrying the local spanwise kinetic energy), periodic x2, the similarity-
profile initial condition.  The statistics classes and the restart read of the app are left out.
Grid size, dt and step count are run-time parameters.
"""
from sympy import cos, sin, exp
from opensbli import *
from opensbli.utilities.katzer_init import Initialise_Katzer
from opensbli.utilities.oblique_shock import ShockConditions
from opensbli.utilities.helperfunctions import substitute_simulation_parameters

ndim = 3
sc1 = "**{'scheme':'Teno'}"
mass = "Eq(Der(rho,t), - Conservative(rhou_j,x_j,%s))" % sc1
momentum = "Eq(Der(rhou_i,t) , -Conservative(rhou_i*u_j + KD(_i,_j)*p,x_j , %s) + Der(tau_i_j,x_j) )" % sc1
energy = "Eq(Der(rhoE,t), - Conservative((p+rhoE)*u_j,x_j, %s) - Der(q_j,x_j) + Der(u_i*tau_i_j ,x_j) )" % sc1
stress_tensor = "Eq(tau_i_j, (mu/Re)*(Der(u_i,x_j)+ Der(u_j,x_i) - (2/3)* KD(_i,_j)* Der(u_k,x_k)))"
heat_flux = "Eq(q_j, (-mu/((gama-1)*Minf*Minf*Pr*Re))*Der(T,x_j))"
substitutions = [stress_tensor, heat_flux]
constants = ["Re", "Pr", "gama", "Minf", "SuthT", "RefT"]
coordinate_symbol = "x"
velocity = "Eq(u_i, rhou_i/rho)"
pressure = "Eq(p, (gama-1)*(rhoE - rho*(1/2)*(KD(_i,_j)*u_i*u_j)))"
speed_of_sound = "Eq(a, (gama*p/rho)**0.5)"
temperature = "Eq(T, p*gama*Minf*Minf/(rho))"
viscosity = "Eq(mu, (T**(1.5)*(1.0+SuthT/RefT)/(T+SuthT/RefT)))"

eq = EinsteinEquation()
base_eqns = [eq.expand(e, ndim, coordinate_symbol, substitutions, constants) for e in [mass, momentum, energy]]
constituent_eqns = [eq.expand(e, ndim, coordinate_symbol, substitutions, constants)
                    for e in [velocity, pressure, speed_of_sound, temperature, viscosity]]

block = SimulationBlock(ndim, block_number=0)
local_dict = {"block": block, "GridVariable": GridVariable, "DataObject": DataObject}
metriceq = MetricsEquation()
metriceq.generate_transformations(ndim, coordinate_symbol, [(False, False), (True, False), (False, False)], 2)

sensor_eqns, sensor_array = ShockSensor().ducros_equations(block, coordinate_symbol, metriceq)
schemes = {}
teno = LLFTeno(6, formulation='adaptive', averaging=RoeAverage([0, 1]), sensor=sensor_array, store_sensor=True)
schemes[teno.name] = teno
cent = StoreSome(4, 'u0 u1 u2')
schemes[cent.name] = cent
rk = RungeKuttaLS(3)
schemes[rk.name] = rk
block.set_discretisation_schemes(schemes)

# the body force of the app, a source in the continuity equation
A, B, xF, yF, bta, omega, dt = symbols('A B xF yF bta omega dt', **{'cls': ConstantObject})
it = block.get_temporal_schemes[0].iteration_number
x0, x1, x2 = symbols('x0 x1 x2', **{'cls': DataObject})
body_force = Eq(DataObject('BF'), A*exp(-((x0-xF)**2+(x1-yF)**2))*cos(bta*x2)*sin(omega*dt*it))
base_eqns[0] = Eq(base_eqns[0].lhs, base_eqns[0].rhs + body_force.lhs)

simulation_eq = SimulationEquations()
constituent = ConstituentRelations()
for e in base_eqns:
    simulation_eq.add_equations(e)
for e in constituent_eqns:
    constituent.add_equations(e)
simulation_eq.apply_metrics(metriceq)
constituent.add_equations(sensor_eqns)
constituent.add_equations(body_force)

boundaries = [[0, 0] for t in range(ndim)]
boundaries[0][0] = InletPressureExtrapolateBC(0, 0, scheme=ReducedAccess())
boundaries[0][1] = ExtrapolationBC(0, 1, order=0, scheme=ReducedAccess())
for con in ["Lx1", "by", "Twall"]:
    local_dict[con] = ConstantObject(con)
CTD.add_constant(ConstantObject('Twall'))
rhoE_wall = parse_expr("Eq(DataObject(rhoE), DataObject(rho)*Twall/(gama*(gama-1.0)*Minf**2.0))", local_dict=local_dict)
boundaries[1][0] = IsothermalWallBC(1, 0, [rhoE_wall], scheme=ReducedAccess())
gamma, xmach = 1.4, 1.5
pre = (1.0, 1.0, 0.00466654053208844, (1.0/(gamma*xmach**2))/(gamma-1.0) + 0.5*(1.0 + 0.00466654053208844**2))
post = ShockConditions(44.6607551, xmach, gamma).conservative_post_shock_conditions(1.0)
top = [parse_expr("Eq(DataObject(rho), Piecewise((%.15f, DataObject(x0)>20.0), (%.15f, True)))" % (post[0], pre[0]), local_dict=local_dict),
       parse_expr("Eq(DataObject(rhou0), Piecewise((%.15f, DataObject(x0)>20.0), (%.15f, True)))" % (post[1], pre[1]), local_dict=local_dict),
       parse_expr("Eq(DataObject(rhou1), Piecewise((%.15f, DataObject(x0)>20.0), (%.15f, True)))" % (post[2], pre[2]), local_dict=local_dict),
       parse_expr("Eq(DataObject(rhoE), Piecewise((%.15f + 0.5*DataObject(rhou2)**2 / DataObject(rho), DataObject(x0)>20.0), "
                  "(%.15f + 0.5*DataObject(rhou2)**2 / DataObject(rho), True)))" % (post[3], pre[3]), local_dict=local_dict)]
boundaries[1][1] = DirichletBC(1, 1, top, scheme=ReducedAccess())
boundaries[2][0] = PeriodicBC(2, 0)
boundaries[2][1] = PeriodicBC(2, 1)
block.set_block_boundaries(boundaries)

gridx0 = parse_expr("Eq(DataObject(x0), block.deltas[0]*block.grid_indexes[0])", local_dict=local_dict)
gridx1 = parse_expr("Eq(DataObject(x1), Lx1*sinh(by*block.deltas[1]*block.grid_indexes[1]/Lx1)/sinh(by))", local_dict=local_dict)
gridx2 = parse_expr("Eq(DataObject(x2), block.deltas[2]*block.grid_indexes[2])", local_dict=local_dict)
initial = Initialise_Katzer([(False, DataObject('x0')), (True, DataObject('x1')), (False, DataObject('x2'))], 50,
                            750.0, 1.5, 202.17, [gridx0, gridx1, gridx2])

h5 = iohdf5(iotype="Write")
h5.add_arrays(simulation_eq.time_advance_arrays)
h5.add_arrays([DataObject('x0'), DataObject('x1'), DataObject('x2'), DataObject('D11'), DataObject('TENO')])
block.setio(h5)
block.set_equations([simulation_eq, constituent, initial, metriceq])
block.discretise()
alg = TraditionalAlgorithmRK(block)
SimulationDataType.set_datatype(Double)
OPSC(alg)
constants = ['gama', 'Minf', 'Pr', 'Re', 'Twall', 'dt', 'niter', 'block0np0', 'block0np1', 'block0np2',
             'Delta0block0', 'Delta1block0', 'Delta2block0', 'SuthT', 'RefT', 'eps', 'Lx1', 'by', 'A', 'bta', 'omega',
             'xF', 'yF', 'teno_a1', 'teno_a2', 'epsilon']
values = ['1.4', '1.5', '0.72', '750.0', '1.3809973268575328', '0.025', '300000', '500', '200', '100',
          '375.0/(block0np0-1)', '140.0/(block0np1-1)', '27.32/(block0np2)', '110.4', '202.17', '1e-30', '140.0',
          '5.0', '2.5e-3', '0.23', '0.1011', '20.0', '4.0', '9.5', '3.5', '1.0e-16']
substitute_simulation_parameters(constants, values)
