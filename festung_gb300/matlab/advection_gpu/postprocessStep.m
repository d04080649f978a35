% advection/postprocessStep.m:54-61; cDisc is read back when output or post-processing needs it.
function problemData = postprocessStep(problemData, nStep)
problemData.isFinished = nStep >= problemData.numSteps;
end % function
