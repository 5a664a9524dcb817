"""Problem script: 3D Taylor-Green vortex with TENO5 fluxes whose cut-off adapts to the modified
Ducros sensor.

Written for this build against the reference's user API: tgv_teno.py with the adaptive cut-off of the
published Katzer script (apps/katzer_SBLI/katzer_SBLI.py:57-65: ShockSensor().ducros_equations added
to the constituent relations, LLFTeno(5, formulation='adaptive', sensor=..., store_sensor=True)) on a
periodic 3D block without metrics.  Constants become run-time parameters.
"""
from opensbli import *
from opensbli.utilities.helperfunctions import substitute_simulation_parameters

ndim = 3
sc1 = "**{'scheme':'Teno'}"
mass = "Eq(Der(rho,t), - Conservative(rhou_j,x_j,%s))" % sc1
momentum = "Eq(Der(rhou_i,t) , -Conservative(rhou_i*u_j + KD(_i,_j)*p,x_j , %s) + Der(tau_i_j,x_j) )" % sc1
energy = "Eq(Der(rhoE,t), - Conservative((p+rhoE)*u_j,x_j, %s) + Der(q_j,x_j) + Der(u_i*tau_i_j ,x_j) )" % sc1
stress_tensor = "Eq(tau_i_j, (1.0/Re)*(Der(u_i,x_j)+ Der(u_j,x_i)- (2/3)* KD(_i,_j)* Der(u_k,x_k)))"
heat_flux = "Eq(q_j, (1.0/((gama-1)*Minf*Minf*Pr*Re))*Der(T,x_j))"
substitutions = [stress_tensor, heat_flux]
constants = ["Re", "Pr", "gama", "Minf"]
coordinate_symbol = "x"
velocity = "Eq(u_i, rhou_i/rho)"
pressure = "Eq(p, (gama-1)*(rhoE - rho*(1/2)*(KD(_i,_j)*u_i*u_j)))"
speed_of_sound = "Eq(a, (gama*p/rho)**0.5)"
temperature = "Eq(T, p*gama*Minf*Minf/(rho))"

eq = EinsteinEquation()
simulation_eq = SimulationEquations()
for base in [mass, momentum, energy]:
    simulation_eq.add_equations(eq.expand(base, ndim, coordinate_symbol, substitutions, constants))
constituent = ConstituentRelations()
for cr in [velocity, pressure, speed_of_sound, temperature]:
    constituent.add_equations(eq.expand(cr, ndim, coordinate_symbol, substitutions, constants))

block = SimulationBlock(ndim, block_number=0)
# the modified Ducros sensor drives the TENO cut-off (apps/katzer_SBLI/katzer_SBLI.py:57-65, no metrics)
SS = ShockSensor()
shock_sensor, sensor_array = SS.ducros_equations(block, coordinate_symbol, None)
constituent.add_equations(shock_sensor)
local_dict = {"block": block, "GridVariable": GridVariable, "DataObject": DataObject}
ics = [
    "Eq(GridVariable(x0), block.deltas[0]*block.grid_indexes[0])",
    "Eq(GridVariable(x1), block.deltas[1]*block.grid_indexes[1])",
    "Eq(GridVariable(x2), block.deltas[2]*block.grid_indexes[2])",
    "Eq(GridVariable(u0),sin(x0)*cos(x1)*cos(x2))",
    "Eq(GridVariable(u1),-cos(x0)*sin(x1)*cos(x2))",
    "Eq(GridVariable(u2), 0.0)",
    "Eq(GridVariable(p), 1.0/(gama*Minf*Minf)+ (1.0/16.0) * (cos(2.0*x0)+cos(2.0*x1))*(2.0 + cos(2.0*x2)))",
    "Eq(GridVariable(r), gama*Minf*Minf*p)",
    "Eq(DataObject(rho), r)",
    "Eq(DataObject(rhou0), r*u0)",
    "Eq(DataObject(rhou1), r*u1)",
    "Eq(DataObject(rhou2), r*u2)",
    "Eq(DataObject(rhoE), p/(gama-1) + 0.5* r *(u0**2+ u1**2 + u2**2))",
]
initial = GridBasedInitialisation()
initial.add_equations([parse_expr(e, local_dict=local_dict) for e in ics])

schemes = {}
teno = LLFTeno(5, formulation='adaptive', averaging=RoeAverage([0, 1]), sensor=sensor_array,
              store_sensor=True)
schemes[teno.name] = teno
cent = Central(4)
schemes[cent.name] = cent
rk = RungeKutta(3)
schemes[rk.name] = rk

boundaries = []
for direction in range(ndim):
    boundaries += [PeriodicBC(direction, 0), PeriodicBC(direction, 1)]
block.set_block_boundaries(boundaries)
h5 = iohdf5(save_every=1000000, iotype="Write")
h5.add_arrays(simulation_eq.time_advance_arrays)
block.setio(h5)
block.set_equations([constituent, simulation_eq, initial])
block.set_discretisation_schemes(schemes)
block.discretise()
alg = TraditionalAlgorithmRK(block)
SimulationDataType.set_datatype(Double)
OPSC(alg)
constants = ['Re', 'gama', 'Minf', 'Pr', 'dt', 'niter', 'block0np0', 'block0np1', 'block0np2',
             'Delta0block0', 'Delta1block0', 'Delta2block0', 'eps', 'TENO_CT', 'teno_a1', 'teno_a2', 'epsilon']
values = ['1600.0', '1.4', '1.25', '0.71', '0.001', '10', '64', '64', '64',
          '2*M_PI/block0np0', '2*M_PI/block0np1', '2*M_PI/block0np2', '1e-15', '1e-5', '10.5', '4.5', '1e-30']
substitute_simulation_parameters(constants, values)
