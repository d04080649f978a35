function problemData = preprocessStep(problemData, nStep) %#ok<INUSD>
end % function
